/*
 * lss_phantom.h — deterministic synthetic volumes for tests and benchmarks.
 *
 * The reference measured on BrainWeb MRI volumes, which are not shipped with
 * it; these generators stand in for them with seeded synthetic phantoms of
 * the same shapes and value ranges.  Every generator uses only integer
 * hashing, IEEE additions, multiplications, divisions and square roots (no
 * libm transcendentals), so x86-64 and aarch64 produce identical bits.
 * Gaussian noise is the Irwin-Hall approximation (sum of 4 uniforms,
 * rescaled to unit variance).
 */
#ifndef LSS_PHANTOM_H
#define LSS_PHANTOM_H

#include <stdint.h>
#include "lss.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One ellipsoid (centre c, semi-axes a) of value fg on background bg, plus
 * noise of std noise_sigma from `seed`. */
lss_status lss_phantom_ellipsoid(int32_t nx, int32_t ny, int32_t nz,
                                 const float* centre3, const float* semi_axes3,
                                 float fg, float bg, float noise_sigma, uint64_t seed,
                                 float* out);

/* Nested ellipsoid shells about the volume centre.  semi_axes holds 3 floats
 * per shell, outermost first; values one float per shell.  Each boundary is
 * displaced by trilinear value noise of amplitude disp_amp voxels on a
 * lattice of spacing `lattice` (seed disp_seed); then a Gaussian blur of
 * sigma blur_sigma (0 or 1 only) is applied, then noise (noise_seed). */
lss_status lss_phantom_shells(int32_t nx, int32_t ny, int32_t nz, int32_t nshells,
                              const float* semi_axes, const float* values, float bg,
                              float disp_amp, int32_t lattice, uint64_t disp_seed,
                              float blur_sigma, float noise_sigma, uint64_t noise_seed,
                              float* out);

/* Union (min) of signed distances to spheres (x, y, z, r per sphere),
 * clamped to [lo, hi]; negative inside. */
lss_status lss_phantom_sdf_spheres(int32_t nx, int32_t ny, int32_t nz, const float* xyzr,
                                   int32_t count, float lo, float hi, float* out);

/* Deterministic uniform draws in [0,1) from (seed, index): used to draw batch
 * shapes and parameters identically on every platform. */
double lss_phantom_uniform(uint64_t seed, uint64_t index);

#ifdef __cplusplus
}
#endif

#endif /* LSS_PHANTOM_H */
