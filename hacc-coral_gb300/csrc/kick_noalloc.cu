// kick_noalloc.cu -- the short-range kick over caller-supplied interaction
// lists with no memory allocation at all.
//
// Some callers cannot allocate device memory while they run: a simulation
// that sizes every buffer up front and forbids allocation inside its time
// loop, code running under a memory pool or arena that owns the whole device,
// or an embedding that must not grow its footprint after start-up.  For them,
// hsr_kick_lists_noalloc evaluates the pair kick with the batched culling
// kernel, keeping the kernel's scratch -- the work items it builds from the
// leaves and the work-queue and statistics counters -- in the fixed array
// below instead of in allocated buffers.  Inputs and outputs are the caller's
// own device arrays.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "hacc_sr.h"
#include "sr_kernels.cuh"

namespace {

// The scratch array: 4 MiB on every device that loads the library, held until
// the process exits.  Layout: three 64-bit counters (work-queue head,
// evaluated pairs, items reserved), an overflow flag, then the work items.
constexpr size_t kScratchBytes = size_t(4) << 20;
constexpr size_t kItemsOffset = 256;
constexpr int64_t kMaxItems = int64_t((kScratchBytes - kItemsOffset) / sizeof(hsr::PairItem));
// Longest list range of one item; longer lists are split over several items.
constexpr int64_t kSplit = 8192;
constexpr int kWarps = 8;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct ScratchHead {
  unsigned long long queue;      // next item to take
  unsigned long long evaluated;  // pairs evaluated after the box test
  unsigned long long reserved;   // items reserved by the builder
  unsigned int overflow;         // set when the items do not fit
};

__device__ __forceinline__ ScratchHead *head(unsigned char *scr) {
  return reinterpret_cast<ScratchHead *>(scr);
}
__device__ __forceinline__ hsr::PairItem *item_at(unsigned char *scr, int64_t i) {
  return reinterpret_cast<hsr::PairItem *>(scr + kItemsOffset) + i;
}

// Work items: each leaf's particles in consecutive groups of up to 32, each
// group against list ranges of at most kSplit entries.
__global__ void k_noalloc_items(unsigned char *scr, const int32_t *leaf_offset,
                                const int32_t *leaf_count, const int64_t *list_begin,
                                const int32_t *list_len, int64_t nleaves) {
  const int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (l >= nleaves) return;
  const int32_t cnt = leaf_count[l], len = list_len[l];
  if (cnt <= 0 || len <= 0) return;
  const int64_t nch = (int64_t(len) + kSplit - 1) / kSplit;
  const int32_t ng = (cnt + 31) / 32;
  const int64_t need = nch * ng;
  const unsigned long long at = atomicAdd(&head(scr)->reserved, (unsigned long long)need);
  if (int64_t(at) + need > kMaxItems) {
    atomicExch(&head(scr)->overflow, 1u);
    return;
  }
  int64_t k = int64_t(at);
  for (int32_t g = 0; g < ng; ++g)
    for (int64_t c = 0; c < nch; ++c) {
      hsr::PairItem it{};
      it.j_begin = list_begin[l] + c * kSplit;
      it.j_len = int32_t(c + 1 < nch ? kSplit : len - c * kSplit);
      it.g_begin = leaf_offset[l] + 32 * g;
      it.g_count = cnt - 32 * g < 32 ? cnt - 32 * g : 32;
      it.flags = nch > 1 ? 1 : 0;
      *item_at(scr, k++) = it;
    }
}

// The batched pair kernel (sr_kernels.cu, k_pairs_batched) with its items and
// counters in the scratch array and groups of consecutive particles.
template <int LAW>
__global__ void __launch_bounds__(32 * kWarps)
    k_noalloc_pairs(unsigned char *scr, const float4 *__restrict__ table,
                    const int32_t *__restrict__ idx,
                    float *__restrict__ vx, float *__restrict__ vy, float *__restrict__ vz,
                    float fcoeff, float rsm2, float rcut2, float rcull2) {
  __shared__ float4 slot[kWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  // items that did not fit: no pair is evaluated, the velocities stay as
  // they are and the host reports the overflow
  if (head(scr)->overflow) return;
  const unsigned long long nitems = head(scr)->reserved;
  unsigned long long evaluated = 0;
  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(&head(scr)->queue, 1ull);
    it = __shfl_sync(full, it, 0);
    if (it >= nitems) break;
    const hsr::PairItem W = *item_at(scr, int64_t(it));
    const bool act = lane < W.g_count;
    const int pi = W.g_begin + (act ? lane : 0);
    const float4 P = table[pi];
    float lox = P.x, hix = P.x, loy = P.y, hiy = P.y, loz = P.z, hiz = P.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lox = fminf(lox, __shfl_xor_sync(full, lox, o));
      hix = fmaxf(hix, __shfl_xor_sync(full, hix, o));
      loy = fminf(loy, __shfl_xor_sync(full, loy, o));
      hiy = fmaxf(hiy, __shfl_xor_sync(full, hiy, o));
      loz = fminf(loz, __shfl_xor_sync(full, loz, o));
      hiz = fmaxf(hiz, __shfl_xor_sync(full, hiz, o));
    }
    float ax = 0.f, ay = 0.f, az = 0.f;
    const int32_t *lst = idx + W.j_begin;
    for (int j0 = 0; j0 < W.j_len; j0 += 32) {
      const int j = j0 + lane;
      const bool ok = j < W.j_len;
      const float4 J = table[lst[ok ? j : 0]];
      const float dx = fmaxf(fmaxf(lox - J.x, J.x - hix), 0.f);
      const float dy = fmaxf(fmaxf(loy - J.y, J.y - hiy), 0.f);
      const float dz = fmaxf(fmaxf(loz - J.z, J.z - hiz), 0.f);
      unsigned keep = __ballot_sync(full, ok && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < rcull2);
      if (!keep) continue;
      evaluated += (unsigned long long)__popc(keep) * (unsigned long long)W.g_count;
      slot[w][lane] = J;
      __syncwarp();
      while (keep) {
        const int b = __ffs(keep) - 1;
        keep &= keep - 1;
        hsr::pair_acc<LAW>(P.x, P.y, P.z, slot[w][b], rsm2, rcut2, ax, ay, az);
      }
      __syncwarp();
    }
    if (act) {
      const float c = (LAW == hsr::LAW_POLY5_STEP16) ? fcoeff : fcoeff * P.w;
      if (W.flags & 1) {
        atomicAdd(vx + pi, c * ax);
        atomicAdd(vy + pi, c * ay);
        atomicAdd(vz + pi, c * az);
      } else {
        vx[pi] += c * ax;
        vy[pi] += c * ay;
        vz[pi] += c * az;
      }
    }
  }
  if (lane == 0 && evaluated) atomicAdd(&head(scr)->evaluated, evaluated);
}

// The device address of g_scratch.  In host code the name g_scratch is only a
// host-side stand-in, not a device address: handing it to a kernel would
// fault (or, where the GPU can reach host memory, silently use the wrong
// memory).  So the first call on each device, with that device current, asks
// the runtime for the real address (set-up) and every call passes that to the
// kernels.  Later calls ask again unless their stream is capturing, so the
// address follows the module if the device's context was reset between calls.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

hsr_status scratch_address(int dev, cudaStream_t s, void **out) {
  if (dev < 0 || dev >= kMaxDevices) return HSR_ERR_UNSUPPORTED;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return HSR_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev] || cap == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return HSR_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return HSR_OK;
}

}  // namespace

extern "C" hsr_status hsr_kick_lists_noalloc(const float *table, int64_t ntab, int64_t n,
                                             const int32_t *leaf_offset, const int32_t *leaf_count,
                                             const int64_t *list_begin, const int32_t *list_len,
                                             int64_t nleaves, const int32_t *list_index,
                                             float *vx, float *vy, float *vz, float fcoeff,
                                             float rsm, float fsrrmax, int32_t law, void *stream) {
  if (nleaves < 0 || n < 0 || ntab < n) return HSR_ERR_ARG;
  if (nleaves == 0) return HSR_OK;
  if (!table || !leaf_offset || !leaf_count || !list_begin || !list_len || !list_index || !vx ||
      !vy || !vz)
    return HSR_ERR_ARG;
  if (reinterpret_cast<uintptr_t>(table) % 16 != 0) return HSR_ERR_ARG;
  if (law != HSR_LAW_POLY6 && law != HSR_LAW_POLY5_STEP16) return HSR_ERR_ARG;
  if (nleaves > kMaxItems) return HSR_ERR_ARG;  // at least one item per leaf
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return HSR_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the scratch address and the launches are the current device's: a stream
  // of another device is refused
  int sdev = -1;
  if (cudaStreamGetDevice(s, &sdev) != cudaSuccess || sdev != dev) return HSR_ERR_ARG;
  void *base = nullptr;
  if (hsr_status st = scratch_address(dev, s, &base)) return st;
  // counters and the overflow flag start at zero on every call (the array
  // keeps the last call's)
  if (cudaMemsetAsync(base, 0, sizeof(ScratchHead), s) != cudaSuccess) return HSR_ERR_CUDA;
  unsigned char *scr = static_cast<unsigned char *>(base);
  k_noalloc_items<<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(scr, leaf_offset, leaf_count,
                                                                   list_begin, list_len, nleaves);
  if (cudaGetLastError() != cudaSuccess) return HSR_ERR_CUDA;
  const float fs2 = fsrrmax * fsrrmax;
  const float rmax = 3.116326355f, r2max = rmax * rmax;
  const float rc2 = law == HSR_LAW_POLY5_STEP16
                        ? fs2
                        : (fs2 < nextafterf(r2max, INFINITY) ? fs2 : nextafterf(r2max, INFINITY));
  const float rcull2 = rc2 * 1.0001f + 1e-6f;
  // persistent grid from the SM count and occupancy alone: the pair kernel
  // reads the item count (and the overflow flag) on the device, and CTAs
  // beyond the work exit at their first queue read
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (law == HSR_LAW_POLY5_STEP16)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_noalloc_pairs<hsr::LAW_POLY5_STEP16>,
                                                  32 * kWarps, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_noalloc_pairs<hsr::LAW_POLY6>,
                                                  32 * kWarps, 0);
  const int64_t ctas = int64_t(sms > 0 ? sms : 1) * (per > 0 ? per : 1);
  const float4 *tab = reinterpret_cast<const float4 *>(table);
  if (law == HSR_LAW_POLY5_STEP16)
    k_noalloc_pairs<hsr::LAW_POLY5_STEP16><<<unsigned(ctas), 32 * kWarps, 0, s>>>(
        scr, tab, list_index, vx, vy, vz, fcoeff, rsm * rsm, rc2, rcull2);
  else
    k_noalloc_pairs<hsr::LAW_POLY6><<<unsigned(ctas), 32 * kWarps, 0, s>>>(
        scr, tab, list_index, vx, vy, vz, fcoeff, rsm * rsm, rc2, rcull2);
  if (cudaGetLastError() != cudaSuccess) return HSR_ERR_CUDA;
  // the overflow flag comes back once the kernels are done (a copy into host
  // stack memory, which waits for the stream)
  ScratchHead h{};
  if (cudaMemcpyAsync(&h, base, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return HSR_ERR_CUDA;
  if (h.overflow) return HSR_ERR_ARG;  // more work items than the fixed array holds
  return HSR_OK;
}
