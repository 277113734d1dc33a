"""bench.py's reference arm (the CPU restatement timed on the host cores)
prints its one-line JSON benchmark record: checked on the CPU at a small
scale.  The arm names the same workload as the GPU arm (the same `config`
dict, built by one function for both), times one whole seeding + run to
convergence, and its process loads the oracle and the input generator but
not the solver library.  The GPU arm prints the same keys plus roofline,
clocks and e2e figures; it runs in the GPU environment only."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Runs the reference arm in a fresh interpreter, then reports which in-tree
# shared libraries that process mapped.
_PROBE = r"""
import io, json, sys, contextlib
sys.argv = ["bench.py", "--impl", "reference", "--steps", "3", "--warmup", "1", "--scale", "0.125"]
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
maps = open("/proc/self/maps").read()
libs = sorted({l.split()[-1].rsplit("/", 1)[-1] for l in maps.splitlines() if l.endswith(".so")})
print(json.dumps({"line": buf.getvalue(), "libs": libs}))
"""


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "-c", _PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    probe = json.loads(r.stdout.strip().splitlines()[-1])
    lines = [ln for ln in probe["line"].splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["metric"] == "active_voxel_updates_per_s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert "to convergence" in cb["sample"] and cb["config1"]["iterations"] == 300
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # The same workload dict as the GPU arm builds.
    sys.path.insert(0, ROOT)
    import bench
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    assert d["config"] == json.loads(json.dumps(bench.workload_config(P.config2(0.125))))
    # Loads the oracle and the generator, not the solver library.
    assert "liboracle.so" in probe["libs"] and "libphantom.so" in probe["libs"], probe["libs"]
    assert "liblss.so" not in probe["libs"], probe["libs"]


def test_oracle_run_covers_the_whole_run_in_segments():
    """Segmenting the timed run does not change the work: any split gives
    the same iterations and updates as one piece, and the same as the
    oracle's own stopping-rule loop."""
    sys.path.insert(0, ROOT)
    import bench
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    from oracle.oracle import NsOracle
    cfg = P.config2(0.125)
    runs = [bench.oracle_run(cfg, 2, parts, warm) for parts, warm in ((1, 0), (4, 2), (20, 3))]
    assert len({(r[0], r[2]) for r in runs}) == 1
    p = cfg["params"]
    o = NsOracle(cfg["image"], threads=2)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    o.set_phi(cfg["phi0"])
    it = o.run(cfg["conv"]["rel"], cfg["conv"]["patience"], cfg["conv"]["max_iterations"])
    assert (o.updates, it) == (runs[0][0], runs[0][2])


def test_kernel_hash_ignores_comments_and_tracks_code(tmp_path, monkeypatch):
    """The DRAM traffic the bench reports is keyed by a hash of the persistent
    kernel's sources without their comments: a comment edit keeps a capture,
    a code edit drops it (the line then reports no traffic until the kernel
    is captured again)."""
    sys.path.insert(0, ROOT)
    import bench

    src = os.path.join(ROOT, "aworkefficientgpualgorithmforlevelsetsegmentation_gb300", "csrc")
    pkg = tmp_path / "aworkefficientgpualgorithmforlevelsetsegmentation_gb300" / "csrc"
    pkg.mkdir(parents=True)
    for f in bench.KERNEL_SOURCES:
        (pkg / f).write_text(open(os.path.join(src, f)).read())
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    h0 = bench.kernel_source_hash()
    first = bench.KERNEL_SOURCES[0]
    text = (pkg / first).read_text()
    (pkg / first).write_text(text + "\n// a comment\n\n")
    assert bench.kernel_source_hash() == h0
    (pkg / first).write_text(text + "\nstatic const int kUnused = 1;\n")
    assert bench.kernel_source_hash() != h0
