"""Raw volume IO through the C ABI: lss_load_volume_raw (the role of the
reference's VolumeLoader::LoadVolumeRaw, code/gpuseg/code/src/VolumeLoader.cpp:
275-457: numVoxels * bytesPerVoxel bytes, x fastest, read in one piece) and
lss_save_mask_raw (the u8 segmentation written as one raw block).

A volume loaded from a raw file must behave exactly like the same array
passed to lss_load_volume: after seeding and stepping, phi, the active list
and the mask agree bit for bit.  Ragged sides (not multiples of the 16-voxel
REF padding or the 8-voxel NS bricks) and every voxel type are covered; the
six integer types in LSS_MODE_REF (the reference's types), f32 and all the
integer types in LSS_MODE_NS.  Errors: a missing file, a file shorter than the
volume, and dimensions whose byte count overflows return status codes."""
import numpy as np
import pytest

import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss

pytestmark = pytest.mark.gpu

SHAPE = (19, 22, 27)  # z, y, x: ragged against 16 and 8

TYPES = {  # dtype: (foreground, background, noise, REF params T, eps)
    np.uint8: (150, 40, 10, 150, 40),
    np.int8: (90, -30, 8, 90, 40),
    np.uint16: (2000, 500, 80, 2000, 300),
    np.int16: (900, -600, 60, 900, 300),
    np.uint32: (70000, 20000, 900, 70000, 9000),
    np.int32: (50000, -40000, 900, 50000, 9000),
    np.float32: (0.8, 0.2, 0.04, 0.8, 0.1),
}


def volume(dtype, seed):
    fg, bg, sd, *_ = TYPES[dtype]
    rng = np.random.default_rng(seed)
    nz, ny, nx = SHAPE
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    inside = ((x - 13) / 9.0) ** 2 + ((y - 11) / 7.0) ** 2 + ((z - 9) / 6.0) ** 2 < 1.0
    v = np.where(inside, fg, bg) + sd * rng.standard_normal(SHAPE)
    info = np.iinfo(dtype) if np.issubdtype(dtype, np.integer) else None
    if info is not None:
        v = np.clip(np.rint(v), info.min, info.max)
    return np.ascontiguousarray(v.astype(dtype))


def run(seg, mode, dtype):
    fg, bg, sd, T, eps = TYPES[dtype]
    if mode == lss.MODE_REF:
        seg.set_parameters(T, eps, 0.15, 0.25)
    else:
        lo, hi = float(min(fg, bg)), float(max(fg, bg))
        scale = hi - lo
        seg.set_parameters(float(fg), 0.25 * scale, 0.8, 0.5)
    seg.initialize_seed((13, 11, 9), 3)
    seg.step(6)
    seg.step(5)
    return seg.read_phi(), seg.active(), seg.get_saveable_segmentation()


CASES = [(lss.MODE_REF, t) for t in TYPES if t is not np.float32] + [(lss.MODE_NS, t) for t in TYPES]


@pytest.mark.parametrize("mode,dtype", CASES, ids=[f"{'ref' if m == 0 else 'ns'}-{np.dtype(t).name}"
                                                   for m, t in CASES])
def test_raw_load_equals_array_load_and_mask_round_trips(tmp_path, mode, dtype):
    v = volume(dtype, 7 + CASES.index((mode, dtype)))
    path = tmp_path / "vol.raw"
    v.tofile(path)
    a = lss.Segmenter(mode)
    a.load_volume(v)
    b = lss.Segmenter(mode)
    b.load_volume_raw(str(path), SHAPE, dtype)
    assert b.shape == a.shape == SHAPE
    pa, la, ma = run(a, mode, dtype)
    pb, lb, mb = run(b, mode, dtype)
    assert np.array_equal(pa, pb)
    assert np.array_equal(la, lb) and la.size > 0
    assert np.array_equal(ma, mb) and ma.any()
    out = tmp_path / "mask.raw"
    b.save_segmentation_raw(str(out))
    back = np.fromfile(out, np.uint8)
    assert back.size == v.size
    assert np.array_equal(back.reshape(SHAPE), mb)


def test_raw_errors(tmp_path):
    s = lss.Segmenter(lss.MODE_REF)
    with pytest.raises(lss.LssError) as e:
        s.load_volume_raw(str(tmp_path / "missing.raw"), SHAPE, np.uint8)
    assert e.value.status == 1 and "cannot open" in str(e.value)
    short = tmp_path / "short.raw"
    volume(np.uint16, 1).ravel()[:-1].tofile(short)  # one voxel short
    with pytest.raises(lss.LssError) as e:
        s.load_volume_raw(str(short), SHAPE, np.uint16)
    assert e.value.status == 1 and "expected" in str(e.value)
    with pytest.raises(lss.LssError) as e:  # byte count overflows 64 bits
        s.load_volume_raw(str(short), (2**31 - 1, 2**31 - 1, 2**31 - 1), np.float32)
    assert e.value.status == 9
    # The engine is still usable and nothing was loaded by the failed calls.
    with pytest.raises(lss.LssError) as e:
        s.step(1)
    assert e.value.status == 2
    with pytest.raises(lss.LssError):  # nothing to save yet
        s.save_segmentation_raw(str(tmp_path / "m.raw"))
    v = volume(np.uint8, 2)
    ok = tmp_path / "ok.raw"
    v.tofile(ok)
    s.load_volume_raw(str(ok), SHAPE, np.uint8)
    s.set_parameters(150, 40, 0.15, 0.25)
    s.initialize_seed((13, 11, 9), 3)
    s.step(3)
    with pytest.raises(lss.LssError) as e:  # unwritable destination
        s.save_segmentation_raw(str(tmp_path / "no_such_dir" / "m.raw"))
    assert e.value.status == 1 and "cannot write" in str(e.value)
