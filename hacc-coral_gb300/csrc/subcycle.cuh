// subcycle.cuh -- device kernels of the sub-cycle around the kick
// (Particles::map1 and Particles::resortParticles, src/cpu/Particles.cxx).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace hsr {

// x += pt * v (the half-stream; pt = prefactor * tau rounded in float).
cudaError_t launch_stream(float *x, float *y, float *z, const float *vx, const float *vy,
                          const float *vz, int64_t n, float pt, cudaStream_t s);
cudaError_t launch_fill(float *p, int64_t n, float v, cudaStream_t s);

// Stable sort of the particles by unit grid cell of an ng[0] x ng[1] x ng[2]
// box, particles outside it last (Particles::resortParticles), applied to the
// eight float arrays (x, y, z, vx, vy, vz, mass, phi in any order), the ids
// and the masks.  *n_inbox receives the in-box count.  scratch needs
// resort_scratch_bytes(n) bytes.  Synchronizes s.
size_t resort_scratch_bytes(int64_t n);
cudaError_t resort_by_cell(int64_t n, const int32_t ng[3], float *const arr_f[8], int64_t *ids,
                           uint16_t *mask, void *scratch, int64_t *n_inbox, cudaStream_t s);

}  // namespace hsr
