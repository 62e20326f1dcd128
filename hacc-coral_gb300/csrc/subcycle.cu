// subcycle.cu -- the sub-cycle around the short-range kick, on the device:
// Particles::map1 (the half-stream) and Particles::resortParticles (the
// stable counting sort by grid cell that precedes every kick), from
// src/cpu/Particles.cxx:732-758 and :402-488.
#include "subcycle.cuh"

#include <algorithm>

#include "rcb_device.cuh"
#include "device_info.cuh"

namespace hsr {

namespace {

// x += pt * v with separate rounding of the product and the sum, as the
// reference's x[i] + prefactor * tau * vx[i] with pt = prefactor * tau.
__global__ void k_stream(float *x, float *y, float *z, const float *vx, const float *vy,
                         const float *vz, int64_t n, float pt) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    x[i] = __fadd_rn(x[i], __fmul_rn(pt, vx[i]));
    y[i] = __fadd_rn(y[i], __fmul_rn(pt, vy[i]));
    z[i] = __fadd_rn(z[i], __fmul_rn(pt, vz[i]));
  }
}

// Cell key of every particle (Particles::array_index with lo = 0, hi = ng):
// (floor(x) * ng1 + floor(y)) * ng2 + floor(z), or Ng when outside the box.
__global__ void k_cell_keys(const float *x, const float *y, const float *z, int64_t n, int32_t ng0,
                            int32_t ng1, int32_t ng2, uint32_t *key, uint32_t *val,
                            unsigned long long *inbox) {
  const uint32_t Ng = uint32_t(ng0) * uint32_t(ng1) * uint32_t(ng2);
  unsigned long long c = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float fx = floorf(x[i]), fy = floorf(y[i]), fz = floorf(z[i]);
    // the reference casts floorf to int; compare in float first so huge or
    // non-finite values land out of the box instead of overflowing the cast
    const bool in = fx >= 0.f && fx < float(ng0) && fy >= 0.f && fy < float(ng1) && fz >= 0.f &&
                    fz < float(ng2);
    uint32_t k = Ng;
    if (in) k = (uint32_t(int(fx)) * uint32_t(ng1) + uint32_t(int(fy))) * uint32_t(ng2) + uint32_t(int(fz));
    key[i] = k;
    val[i] = uint32_t(i);
    c += in;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(inbox, c);
}

// ---- stable LSD radix sort of (key, value), 8-bit digits -------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixPer = 16;
constexpr int kRadixTile = kRadixThreads * kRadixPer;  // elements per block

// hist[d * nblocks + b]: elements of block b with digit d.
__global__ void __launch_bounds__(kRadixThreads)
    k_radix_hist(const uint32_t *key, int64_t n, int shift, int64_t nblocks, int64_t *hist) {
  __shared__ int h[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int64_t b = blockIdx.x;
  const int64_t base = b * kRadixTile;
  for (int k = threadIdx.x; k < kRadixTile; k += blockDim.x) {
    const int64_t i = base + k;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 0xff], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[int64_t(d) * nblocks + b] = h[d];
}

// Stable scatter: warp w of block b takes the block's elements
// [w * 512, (w + 1) * 512) in order, 32 at a time; ranks among equal digits
// follow the element order (lane order inside a step, warp order across).
__global__ void __launch_bounds__(kRadixThreads)
    k_radix_scatter(const uint32_t *key, const uint32_t *val, int64_t n, int shift,
                    int64_t nblocks, const int64_t *offs, uint32_t *okey, uint32_t *oval) {
  __shared__ int wh[kRadixWarps][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int d = lane; d < 256; d += 32) wh[w][d] = 0;
  __syncwarp();
  const int64_t b = blockIdx.x;
  const int64_t base = b * kRadixTile + int64_t(w) * (kRadixTile / kRadixWarps);
  constexpr int kSteps = kRadixTile / kRadixWarps / 32;
  // phase 1: per-warp digit counts
  for (int s = 0; s < kSteps; ++s) {
    const int64_t i = base + s * 32 + lane;
    if (i < n) atomicAdd(&wh[w][(key[i] >> shift) & 0xff], 1);
  }
  __syncthreads();
  // exclusive prefix over warps per digit, plus the block's global offset
  for (int d = threadIdx.x; d < 256; d += blockDim.x) {
    int64_t run = offs[int64_t(d) * nblocks + b];
    for (int q = 0; q < kRadixWarps; ++q) {
      const int c = wh[q][d];
      wh[q][d] = int(run - offs[int64_t(d) * nblocks + b]);
      run += c;
    }
  }
  __syncthreads();
  // phase 2: ranks in order
  for (int s = 0; s < kSteps; ++s) {
    const int64_t i = base + s * 32 + lane;
    const bool ok = i < n;
    const uint32_t k = ok ? key[i] : 0u;
    const int d = ok ? int((k >> shift) & 0xff) : 256 + lane;  // distinct dummy digits
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    int start = 0;
    if (ok) start = wh[w][d];
    __syncwarp();
    if (ok && lane == leader) wh[w][d] = start + __popc(peers);
    __syncwarp();
    if (ok) {
      const int64_t dst = offs[int64_t(d) * nblocks + b] + start + rank;
      okey[dst] = k;
      oval[dst] = val[i];
    }
  }
}

template <typename T>
__global__ void k_permute(const T *__restrict__ in, const uint32_t *__restrict__ perm, T *out,
                          int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = in[perm[i]];
}

__global__ void k_fill_f32(float *p, int64_t n, float v) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

inline unsigned grid_of(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  return unsigned(std::max<int64_t>(1, std::min<int64_t>(b, int64_t(sm_count()) * 32)));
}

}  // namespace

cudaError_t launch_stream(float *x, float *y, float *z, const float *vx, const float *vy,
                          const float *vz, int64_t n, float pt, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_stream<<<grid_of(n), 256, 0, s>>>(x, y, z, vx, vy, vz, n, pt);
  return cudaGetLastError();
}

cudaError_t launch_fill(float *p, int64_t n, float v, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_fill_f32<<<grid_of(n), 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

size_t resort_scratch_bytes(int64_t n) {
  const int64_t nblocks = (n + kRadixTile - 1) / kRadixTile;
  const int64_t h = 256 * std::max<int64_t>(nblocks, 1);
  size_t b = 4 * size_t(std::max<int64_t>(n, 1)) * 4;          // key, val, key', val'
  b += size_t(h) * 8 * 2;                                       // histograms, offsets
  b += size_t(scan_tmp_size(h)) * 8 + 4096;
  b += size_t(std::max<int64_t>(n, 1)) * 8 + 256;               // staging for one array
  return b;
}

cudaError_t resort_by_cell(int64_t n, const int32_t ng[3], float *const arr_f[8], int64_t *ids,
                           uint16_t *mask, void *scratch, int64_t *n_inbox, cudaStream_t s) {
  if (n <= 0) {
    *n_inbox = 0;
    return cudaSuccess;
  }
  const int64_t nblocks = (n + kRadixTile - 1) / kRadixTile;
  const int64_t h = 256 * nblocks;
  char *p = static_cast<char *>(scratch);
  auto take = [&](size_t bytes) {
    char *q = p;
    p += (bytes + 255) & ~size_t(255);
    return q;
  };
  uint32_t *key = reinterpret_cast<uint32_t *>(take(size_t(n) * 4));
  uint32_t *val = reinterpret_cast<uint32_t *>(take(size_t(n) * 4));
  uint32_t *key2 = reinterpret_cast<uint32_t *>(take(size_t(n) * 4));
  uint32_t *val2 = reinterpret_cast<uint32_t *>(take(size_t(n) * 4));
  int64_t *hist = reinterpret_cast<int64_t *>(take(size_t(h) * 8));
  int64_t *offs = reinterpret_cast<int64_t *>(take(size_t(h) * 8));
  int64_t *tmp = reinterpret_cast<int64_t *>(take(size_t(scan_tmp_size(h)) * 8));
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(take(64));
  char *stage = take(size_t(n) * 8);
  cudaError_t e = cudaMemsetAsync(cnt, 0, 8, s);
  if (e != cudaSuccess) return e;
  k_cell_keys<<<grid_of(n), 256, 0, s>>>(arr_f[0], arr_f[1], arr_f[2], n, ng[0], ng[1], ng[2], key,
                                         val, cnt);
  const uint64_t Ng = uint64_t(ng[0]) * uint64_t(ng[1]) * uint64_t(ng[2]);
  int bits = 1;
  while ((uint64_t(1) << bits) <= Ng) ++bits;
  for (int shift = 0; shift < bits; shift += 8) {
    k_radix_hist<<<unsigned(nblocks), kRadixThreads, 0, s>>>(key, n, shift, nblocks, hist);
    e = exclusive_scan_i64(hist, offs, h, nullptr, tmp, s);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<unsigned(nblocks), kRadixThreads, 0, s>>>(key, val, n, shift, nblocks, offs,
                                                                key2, val2);
    std::swap(key, key2);
    std::swap(val, val2);
  }
  // apply the permutation to the ten arrays
  float *sf = reinterpret_cast<float *>(stage);
  for (int a = 0; a < 8; ++a) {
    k_permute<float><<<grid_of(n), 256, 0, s>>>(arr_f[a], val, sf, n);
    e = cudaMemcpyAsync(arr_f[a], sf, size_t(n) * 4, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  int64_t *si = reinterpret_cast<int64_t *>(stage);
  k_permute<int64_t><<<grid_of(n), 256, 0, s>>>(ids, val, si, n);
  e = cudaMemcpyAsync(ids, si, size_t(n) * 8, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  uint16_t *sm = reinterpret_cast<uint16_t *>(stage);
  k_permute<uint16_t><<<grid_of(n), 256, 0, s>>>(mask, val, sm, n);
  e = cudaMemcpyAsync(mask, sm, size_t(n) * 2, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  unsigned long long h_cnt = 0;
  e = cudaMemcpyAsync(&h_cnt, cnt, 8, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  *n_inbox = int64_t(h_cnt);
  return cudaGetLastError();
}

}  // namespace hsr
