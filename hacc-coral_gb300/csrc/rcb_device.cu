// rcb_device.cu -- RCB tree, interaction lists and batched work items built on
// the GPU (see rcb_device.cuh for the method).
#include "rcb_device.cuh"
#include "device_info.cuh"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

namespace hsr {

namespace {

// ---- exactly rounded float helpers: never fused, as the reference rounds ----
__device__ __forceinline__ float fmul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float smin_(float a, float b) { return (b < a) ? b : a; }
// ((a*a) + (b*b)) + (c*c)
__device__ __forceinline__ float norm2_(float a, float b, float c) {
  return fadd_(fadd_(fmul_(a, a), fmul_(b, b)), fmul_(c, c));
}

__host__ __device__ __forceinline__ int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

// Exponent of the lowest set bit of a float (INT_MAX for zero, INT_MIN for
// inf/NaN).  A sum of terms that are all multiples of 2^e is exact in double,
// in any order, while the sum of magnitudes stays below 2^(53 + e).
__device__ __forceinline__ int lsb_exp(float t) {
  const uint32_t b = __float_as_uint(t) & 0x7fffffffu;
  if (b == 0) return INT_MAX;
  int e = int(b >> 23);
  if (e == 255) return INT_MIN;
  uint32_t m = b & 0x7fffffu;
  if (e == 0) e = 1;
  else m |= 0x800000u;
  return e - 150 + (__ffs(int(m)) - 1);
}

constexpr int kChunk = 4096;        // elements per statistics / partition chunk
constexpr int kChunkThreads = 256;  // threads per chunk (16 elements each)
constexpr int kWalkStack = 256;     // DFS stack of the list walk
constexpr int kNodeMax = 16384;     // largest node the one-block partition takes
constexpr int kChainSteps = 32;     // chain steps before the one-block partition jumps pointers
constexpr int kPlainSteps = 4;      // single chain steps before the chunk partition jumps runs

enum { C_NCHUNK = 0, C_NSPLIT = 1, C_NFALLBACK = 2, C_NLEAF = 3, C_NSEG = 4, C_NENT = 5,
       C_PAIRS = 6, C_PADDED = 7, C_NITEMS = 8, C_MAXLEN = 9, C_TDONE1 = 10, C_TDONE2 = 11,
       C_NTIGHT = 12, C_SEGOVF = 13, C_MAXCNT = 14, C_ERR = 15, C_BUCKET = 16, C_FILL = 48,
       C_SUBFB = 80, C_CHAINS = 81, C_COUNT = 82 };

// Segments a leaf's walk can leave in its own region of the one-pass walk;
// a leaf with more sends the build to the counting walk and a second pass.
constexpr int kLocalSegs = 64;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---------------------------------------------------------------------------
// Scan
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int64_t kScanBlock = kScanThreads * kScanPer;

__global__ void __launch_bounds__(kScanThreads)
    k_scan_block(const int64_t *in, int64_t *out, int64_t n, int64_t *bsum, int64_t *total) {
  __shared__ int64_t wsum[32];
  const int64_t base = int64_t(blockIdx.x) * kScanBlock + int64_t(threadIdx.x) * kScanPer;
  int64_t v[kScanPer];
  int64_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    t += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  const int64_t excl = x - t + (warp > 0 ? wsum[warp - 1] : 0);
  int64_t run = excl;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == kScanThreads - 1) {
    bsum[blockIdx.x] = run;
    if (total) *total = run;  // single-block scans only (the caller passes it then)
  }
}

__global__ void k_scan_add(int64_t *out, int64_t n, const int64_t *boff) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] += boff[i / kScanBlock];
}


}  // namespace

int64_t scan_tmp_size(int64_t n) {
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  return nb <= 1 ? 2 : nb + 1 + scan_tmp_size(nb);
}

cudaError_t exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *total,
                               int64_t *tmp, cudaStream_t s) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(int64_t), s);
    return cudaSuccess;
  }
  const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_block<<<unsigned(nb), kScanThreads, 0, s>>>(in, out, n, tmp, nb == 1 ? total : nullptr);
  if (nb == 1) return cudaGetLastError();
  // scan the block sums in place, then add them
  cudaError_t e = exclusive_scan_i64(tmp, tmp, nb, total, tmp + nb + 1, s);
  if (e != cudaSuccess) return e;
  k_scan_add<<<unsigned((n + 255) / 256), 256, 0, s>>>(out, n, tmp);
  return cudaGetLastError();
}

namespace {

// ---------------------------------------------------------------------------
// Level kernels
// ---------------------------------------------------------------------------

// Number of chunks of each node of the level [nb, ne).
__global__ void k_chunk_counts(const DNode *nodes, int32_t nb, int32_t ne, int64_t *cnt) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (nb + i < ne) cnt[i] = (int64_t(nodes[nb + i].count) + kChunk - 1) / kChunk;
}

__global__ void k_chunk_fill(const DNode *nodes, int32_t nb, int32_t ne, const int64_t *base,
                             int32_t *chunk_node) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (nb + i >= ne) return;
  const int64_t c = (int64_t(nodes[nb + i].count) + kChunk - 1) / kChunk;
  for (int64_t k = 0; k < c; ++k) chunk_node[base[i] + k] = nb + i;
}

// Exclusive scan over one block of kScanThreads threads, kScanPer values each
// (v in, out out); returns the block total to every thread.
__device__ __forceinline__ int64_t block_exclusive_scan(const int64_t (&v)[kScanPer],
                                                        int64_t (&out)[kScanPer]) {
  __shared__ int64_t wsum[32];
  int64_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) t += v[k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  int64_t run = x - t + (warp > 0 ? wsum[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    out[k] = run;
    run += v[k];
  }
  return wsum[31];
}

// Levels of at most kScanBlock nodes, in one block: the chunks of every node
// (k_chunk_counts, the scan and k_chunk_fill), the total into *nchunk.
__global__ void __launch_bounds__(kScanThreads)
    k_chunk_setup_small(const DNode *nodes, int32_t nb, int32_t ne, int64_t *base,
                        int32_t *chunk_node, int64_t *counters) {
  int64_t c[kScanPer], b[kScanPer];
  const int32_t i0 = int32_t(threadIdx.x) * kScanPer;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k)
    c[k] = nb + i0 + k < ne ? (int64_t(nodes[nb + i0 + k].count) + kChunk - 1) / kChunk : 0;
  const int64_t total = block_exclusive_scan(c, b);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (nb + i0 + k >= ne) break;
    base[i0 + k] = b[k];
    for (int64_t q = 0; q < c[k]; ++q) chunk_node[b[k] + q] = nb + i0 + k;
  }
  if (threadIdx.x == 0) {
    counters[C_NCHUNK] = total;
    counters[C_NFALLBACK] = 0;  // the level's centre-of-mass lists start empty
    counters[C_NTIGHT] = 0;
    counters[C_MAXCNT] = 0;     // the next level's largest node, from the children
    counters[C_CHAINS] = 0;     // the level's queue of long swap chains
  }
}

// Child s (0 left, 1 right) of split node N, as four 16-byte stores.
__device__ __forceinline__ void write_child(DNode &dst, const DNode &N, int s) {
  DNode C;
  C.count = s == 0 ? N.nleft : N.count - N.nleft;
  C.offset = s == 0 ? N.offset : N.offset + N.nleft;
  C.cl = C.cr = 0;
  for (int d = 0; d < 3; ++d) {
    C.xmin[d] = N.xmin[d];
    C.xmax[d] = N.xmax[d];
    C.xc[d] = 0.f;
  }
  C.tdr = 0.f;
  C.split_dim = -1;
  C.nleft = 0;
  static_assert(sizeof(DNode) == 64, "DNode is four 16-byte words");
  const int4 *src = reinterpret_cast<const int4 *>(&C);
  int4 *out = reinterpret_cast<int4 *>(&dst);
#pragma unroll
  for (int w = 0; w < 4; ++w) out[w] = src[w];
}

// Levels of at most kScanBlock nodes, in one block: k_split_flags, the scan
// and k_children; the number of split nodes into *nsplit.
__global__ void __launch_bounds__(kScanThreads)
    k_children_small(DNode *nodes, int32_t nb, int32_t ne, int64_t *nsplit, int64_t *maxcnt) {
  int64_t f[kScanPer], r[kScanPer];
  unsigned m = 0;  // largest child count of this thread's nodes
  const int32_t i0 = int32_t(threadIdx.x) * kScanPer;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    f[k] = 0;
    if (nb + i0 + k < ne) {
      const DNode &N = nodes[nb + i0 + k];
      f[k] = (N.split_dim >= 0 && N.nleft > 0 && N.nleft < N.count) ? 1 : 0;
    }
  }
  const int64_t total = block_exclusive_scan(f, r);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (nb + i0 + k >= ne) break;
    DNode &N = nodes[nb + i0 + k];
    if (!f[k]) {
      N.cl = N.cr = 0;
      continue;
    }
    const int32_t cl = ne + 2 * int32_t(r[k]), cr = cl + 1;
    N.cl = cl;
    N.cr = cr;
    m = max(m, unsigned(max(N.nleft, N.count - N.nleft)));
    // one block writes every child: whole 16-byte words, not field by field
    for (int s = 0; s < 2; ++s) write_child(nodes[s == 0 ? cl : cr], N, s);
  }
  if (threadIdx.x == 0) *nsplit = total;
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(reinterpret_cast<unsigned long long *>(maxcnt), m);
}

struct ChunkRange {
  int32_t node, begin, len, local;  // local: first element's position inside the node
};

__device__ __forceinline__ ChunkRange chunk_range(const DNode *nodes, const int32_t *chunk_node,
                                                  const int64_t *chunk_base, int32_t nb,
                                                  int64_t chunk) {
  ChunkRange r;
  r.node = chunk_node[chunk];
  const DNode &N = nodes[r.node];
  const int64_t c = chunk - chunk_base[r.node - nb];
  r.local = int32_t(c * kChunk);
  r.begin = N.offset + r.local;
  r.len = min(kChunk, N.count - r.local);
  return r;
}

// Exact sums in 128-bit fixed point.  A float term t is the integer
// t 2^-kFix in units of 2^kFix: exact when t's least significant bit is at
// least 2^kFix, truncated toward zero otherwise (an error below one unit per
// term, counted in the bound).  Terms below 2^14 convert in hardware
// (t 2^48 < 2^62 fits an int64); larger ones take a shift, and terms of
// 2^46 or more flag the chunk (its node takes the sequential sum), which keeps
// a sum of 2^31 terms below 2^125.  Integer adds avoid the FP64 pipe, which
// runs at a small fraction of the FP32 rate on this part.
constexpr int kFix = -48;
constexpr int kFixMaxShift = 70;  // |t| < 2^(70 + 24 + kFix) = 2^46

// Adds t 2^-kFix to acc; ors |t 2^-kFix| into bits (its lowest set bit is the
// least significant bit of all terms, when none is truncated).  |t| < 2^14
// takes a 64-bit shift on the integer pipe; larger terms the 128-bit one.
// (Conversions to and from 64-bit types run on the FP64 pipe, slow here.)
__device__ __forceinline__ void fix_add(__int128 &acc, unsigned __int128 &bits, float t,
                                        bool &overflow, bool &trunc) {
  const uint32_t b = __float_as_uint(t);
  const uint32_t a = b & 0x7fffffffu;
  if (a == 0) return;
  int e = int(a >> 23);
  uint32_t m = a & 0x7fffffu;
  if (e == 0) e = 1;
  else m |= 0x800000u;
  const int sh = e - 150 - kFix;
  unsigned __int128 v;
  if (sh >= 0 && sh <= 39) {
    v = (unsigned __int128)((unsigned long long)m << sh);
  } else if (sh > 39) {
    if (sh > kFixMaxShift || e == 255) overflow = true;
    v = (unsigned __int128)m << min(sh, kFixMaxShift);
  } else {
    const int r = -sh;
    const uint32_t kept = r < 32 ? m >> r : 0u;
    if ((r < 32 ? (kept << r) : 0u) != m) trunc = true;
    v = kept;
  }
  bits |= v;
  acc += (b >> 31) ? -__int128(v) : __int128(v);
}

__device__ __forceinline__ int lsb_of(unsigned __int128 v) {
  const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
  if (lo) return __ffsll((long long)lo) - 1;
  if (hi) return 64 + __ffsll((long long)hi) - 1;
  return -1;
}

// The same sum on the integer pipe.  A term t 2^-kFix with 0 <= shift <= 34
// (2^-24 <= |t| < 2^10, the common case) is m << shift < 2^58, added to a
// signed 64-bit partial sum; fold() moves the partial sum into the 128-bit
// sum (four 32-bit limbs, two's complement, least significant first) and is
// called at least every kFoldTerms adds, so the partial sum stays below 2^62.
// Other terms take fix_add's wide path straight into the limbs.
// lsb: the least significant set bit over the terms' magnitudes (in units of
// 2^kFix), INT_MAX while no term has one.
constexpr int kFoldTerms = 16;
struct FixAcc {
  uint32_t l[4];  // the sum
  long long acc;  // fast-path terms since the last fold
  int lsb;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int k = 0; k < 4; ++k) l[k] = 0u;
    acc = 0;
    lsb = INT_MAX;
  }
  __device__ __forceinline__ void add_limbs(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3) {
    asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.cc.u32 %2, %2, %6;\n\t"
        "addc.u32 %3, %3, %7;"
        : "+r"(l[0]), "+r"(l[1]), "+r"(l[2]), "+r"(l[3])
        : "r"(v0), "r"(v1), "r"(v2), "r"(v3));
  }
  __device__ __forceinline__ void fold() {
    const uint32_t sx = uint32_t(acc >> 63);  // sign extension: 0 or all ones
    add_limbs(uint32_t(acc), uint32_t((unsigned long long)acc >> 32), sx, sx);
    acc = 0;
  }
  __device__ __forceinline__ void add(float t, bool &overflow, bool &trunc) {
    const uint32_t bb = __float_as_uint(t);
    const uint32_t a = bb & 0x7fffffffu;
    if (a == 0) return;
    int e = int(a >> 23);
    uint32_t m = a & 0x7fffffu;
    if (e == 0) e = 1;
    else m |= 0x800000u;
    const int sh = e - 150 - kFix;
    if (unsigned(sh) <= 34u) {
      lsb = min(lsb, sh + __ffs(int(m)) - 1);  // m != 0 here
      const long long v = (long long)((unsigned long long)m << sh);
      acc += (bb >> 31) ? -v : v;
    } else {
      __int128 w = 0;
      unsigned __int128 wb = 0;
      fix_add(w, wb, t, overflow, trunc);
      if (wb) lsb = min(lsb, lsb_of(wb));
      const unsigned __int128 u = (unsigned __int128)w;  // +/- v in two's complement
      add_limbs(uint32_t(u), uint32_t(u >> 32), uint32_t(u >> 64), uint32_t(u >> 96));
    }
  }
  // the 128-bit sum (after a fold)
  __device__ __forceinline__ __int128 sum() const {
    const unsigned __int128 u = ((unsigned __int128)l[3] << 96) | ((unsigned __int128)l[2] << 64) |
                                ((unsigned __int128)l[1] << 32) | (unsigned __int128)l[0];
    return __int128(u);
  }
};

__device__ __forceinline__ __int128 shfl_xor_i128(__int128 v, int o) {
  const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
  const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o);
  const unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o);
  return (__int128(h2) << 64) | __int128(l2);
}

// Correctly rounded double of v 2^kFix: the top 63 bits of |v| with the
// rest folded into a sticky bit, rounded once by the conversion.
__device__ double fix_to_double(__int128 v) {
  const bool neg = v < 0;
  const unsigned __int128 u = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long hi = (unsigned long long)(u >> 64), lo = (unsigned long long)u;
  const int bits = hi ? 128 - __clzll((long long)hi) : (lo ? 64 - __clzll((long long)lo) : 0);
  const int k = bits > 63 ? bits - 63 : 0;
  unsigned long long m = (unsigned long long)(u >> k);
  if (k > 0 && (u & ((((unsigned __int128)1) << k) - 1)) != 0) m |= 1ull;
  const double r = ldexp(__ull2double_rn(m), k + kFix);
  return neg ? -r : r;
}

// Layout of a chunk's partial record (in 8-byte words): sums of the terms
// (x, y, z, m) as 4 x int128, upper bounds of the sums of |terms| (4 doubles),
// the bounding box (6 floats), the least significant exponents (4 ints) and
// an overflow flag.
constexpr int kPartWords = 18;

// The chunk kernels run a block per chunk, or (WM, on deep levels where
// nodes are small) a warp per chunk, 8 chunks per block.
#define CHUNK_PROLOGUE                                                                  \
  const int lane_ = threadIdx.x & 31;                                                 \
  const int64_t chunk =                                                               \
      WM ? int64_t(blockIdx.x) * (kChunkThreads / 32) + (threadIdx.x >> 5) : int64_t(blockIdx.x); \
  const int tid = WM ? lane_ : int(threadIdx.x);                                      \
  constexpr int NT = WM ? 32 : kChunkThreads;                                         \
  (void)lane_;                                                                        \
  (void)tid;                                                                          \
  (void)NT;                                                                           \
  if (chunk >= *nchunk) return;

// Partial sums of one chunk and its bounding box.  Fixed thread-to-element
// map and reduction tree.
template <bool WM>
__global__ void __launch_bounds__(kChunkThreads, 4)
    k_stats_partial(const float4 *__restrict__ pos, const DNode *nodes,
                    const int32_t *chunk_node, const int64_t *chunk_base, int32_t nb,
                    const int64_t *nchunk, double *part) {
  CHUNK_PROLOGUE
  const ChunkRange R = chunk_range(nodes, chunk_node, chunk_base, nb, chunk);
  __int128 s[4] = {0, 0, 0, 0};
  float fa[4] = {0.f, 0.f, 0.f, 0.f};
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool ovf = false;
  bool trn[4] = {false, false, false, false};
  // four loads in flight per thread; the elements are then taken in the same
  // order as one at a time
  constexpr int kU = 2;
  FixAcc fx[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) fx[q].zero();
  int it = 0;
  for (int k0 = tid; k0 < R.len; k0 += NT * kU, ++it) {
    float4 pu[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (k0 + u * NT < R.len) pu[u] = pos[R.begin + k0 + u * NT];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (k0 + u * NT >= R.len) break;
      const float4 p = pu[u];
      const float w = p.w;
      const float t[4] = {fmul_(w, p.x), fmul_(w, p.y), fmul_(w, p.z), w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        fx[q].add(t[q], ovf, trn[q]);
        fa[q] = __fadd_ru(fa[q], fabsf(t[q]));
      }
      lo[0] = fminf(lo[0], p.x); hi[0] = fmaxf(hi[0], p.x);
      lo[1] = fminf(lo[1], p.y); hi[1] = fmaxf(hi[1], p.y);
      lo[2] = fminf(lo[2], p.z); hi[2] = fmaxf(hi[2], p.z);
    }
    if ((it + 1) % (kFoldTerms / kU) == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) fx[q].fold();
    }
  }
  int lsb[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    fx[q].fold();
    s[q] = fx[q].sum();
    lsb[q] = __reduce_min_sync(0xffffffffu, fx[q].lsb);
  }
  double a[4];
  int emin[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) {
      s[q] += shfl_xor_i128(s[q], o);
      fa[q] = __fadd_ru(fa[q], __shfl_xor_sync(0xffffffffu, fa[q], o));
    }
    a[q] = double(fa[q]);
    const bool tq = __any_sync(0xffffffffu, trn[q]);
    // least significant exponent of the warp's terms; below kFix if any term
    // lost bits to the truncation, INT_MAX if all are zero
    emin[q] = tq ? kFix - 1 : (lsb[q] == INT_MAX ? INT_MAX : kFix + lsb[q]);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = warp_min(lo[d]);
    hi[d] = warp_max(hi[d]);
  }
  const bool wovf = __any_sync(0xffffffffu, ovf);
  if (WM) {
    if (lane_ == 0) {
      double *o = part + chunk * kPartWords;
      __int128 *os = reinterpret_cast<__int128 *>(o);
      for (int q = 0; q < 4; ++q) os[q] = s[q];
      for (int q = 0; q < 4; ++q) o[8 + q] = a[q];
      float *ob = reinterpret_cast<float *>(o + 12);
      for (int d = 0; d < 3; ++d) {
        ob[d] = lo[d];
        ob[3 + d] = hi[d];
      }
      int *oe = reinterpret_cast<int *>(o + 15);
      for (int q = 0; q < 4; ++q) oe[q] = emin[q];
      oe[4] = wovf ? 1 : 0;
    }
    return;
  }
  __shared__ __int128 shs[kChunkThreads / 32][4];
  __shared__ double sha[kChunkThreads / 32][4];
  __shared__ float shb[kChunkThreads / 32][6];
  __shared__ int she[kChunkThreads / 32][5];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    for (int q = 0; q < 4; ++q) {
      shs[warp][q] = s[q];
      sha[warp][q] = a[q];
      she[warp][q] = emin[q];
    }
    for (int d = 0; d < 3; ++d) {
      shb[warp][d] = lo[d];
      shb[warp][3 + d] = hi[d];
    }
    she[warp][4] = wovf ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __int128 ts[4];
    double ta[4];
    float tb[6];
    int te[5];
    for (int q = 0; q < 4; ++q) {
      ts[q] = shs[0][q];
      ta[q] = sha[0][q];
      te[q] = she[0][q];
    }
    for (int d = 0; d < 6; ++d) tb[d] = shb[0][d];
    te[4] = she[0][4];
    for (int w = 1; w < kChunkThreads / 32; ++w) {
      for (int q = 0; q < 4; ++q) {
        ts[q] += shs[w][q];
        ta[q] += sha[w][q];
        te[q] = min(te[q], she[w][q]);
      }
      for (int d = 0; d < 3; ++d) {
        tb[d] = fminf(tb[d], shb[w][d]);
        tb[3 + d] = fmaxf(tb[3 + d], shb[w][3 + d]);
      }
      te[4] |= she[w][4];
    }
    double *o = part + chunk * kPartWords;
    __int128 *os = reinterpret_cast<__int128 *>(o);
    for (int q = 0; q < 4; ++q) os[q] = ts[q];
    for (int q = 0; q < 4; ++q) o[8 + q] = ta[q];
    float *ob = reinterpret_cast<float *>(o + 12);
    for (int d = 0; d < 6; ++d) ob[d] = tb[d];
    int *oe = reinterpret_cast<int *>(o + 15);
    for (int q = 0; q < 5; ++q) oe[q] = te[q];
  }
}

// Float that the reference's (float)(sx / sm) gives, if the bounds decide it.
// sx, sm: the sums computed here; bx, bm: bounds on |reference sum - sum here|.
__device__ bool certify(double sx, double bx, double sm, double bm, float *out) {
  const double xl = sx - bx, xh = sx + bx, ml = sm - bm, mh = sm + bm;
  if (!(ml > 0.0) || !isfinite(xl) || !isfinite(xh) || !isfinite(mh)) return false;
  const double q0 = __ddiv_rd(xl, mh), q1 = __ddiv_rd(xl, ml), q2 = __ddiv_ru(xh, mh),
               q3 = __ddiv_ru(xh, ml);
  double lo = fmin(fmin(q0, q1), fmin(q2, q3));
  double hi = fmax(fmax(q0, q1), fmax(q2, q3));
  // the reference rounds its quotient to double once more
  lo -= fabs(lo) * 0x1p-51;
  hi += fabs(hi) * 0x1p-51;
  const float fl = __double2float_rn(lo), fh = __double2float_rn(hi);
  if (fl != fh) return false;
  *out = fl;
  return true;
}

// Sets a node's bounding box and, where decided, its centre of mass from the
// reduced sums; lists it for the tight certification otherwise.
// The node's box, split axis and (where the bounds decide it) centre of mass
// from the reduced sums; false when the centre of mass is left undecided.
__device__ bool decide_node(DNode &N, const __int128 *s, double *a, const float *lo,
                            const float *hi, const int *emin, bool ovf, int32_t force_fallback,
                            int32_t nd) {
  for (int d = 0; d < 3; ++d) {
    N.xmin[d] = lo[d];
    N.xmax[d] = hi[d];
  }
  // leaf by size, or the split axis: the longest box edge, ties to the later
  // axis (RCBForceTree.cxx:837-852); it needs the box only, not the centre
  N.nleft = 0;
  if (N.count <= nd) {
    N.split_dim = -1;
  } else {
    const float l0 = fsub_(N.xmax[0], N.xmin[0]), l1 = fsub_(N.xmax[1], N.xmin[1]),
                l2 = fsub_(N.xmax[2], N.xmin[2]);
    N.split_dim = (l0 > l1 && l0 > l2) ? 0 : (l1 > l2 ? 1 : 2);
  }
  // Sums of |terms|: float partials rounded up, added in double; the factor
  // covers the double additions' rounding.
  for (int q = 0; q < 4; ++q) a[q] *= 1.0 + 0x1p-30;
  const double n = double(N.count);
  // The reference's sequential sum lies within (n - 1) u sum|terms| of the
  // exact sum, to first order; 2 (n + 64) u covers the rest.  This sum is
  // exact except for the truncation of terms with bits below 2^kFix (under
  // 2^kFix each) and its rounding to double.
  const double g = 2.0 * (n + 64.0) * 0x1p-53;
  double sd[4];
  bool exact_ok[4];
  for (int q = 0; q < 4; ++q) {
    sd[q] = fix_to_double(s[q]);
    // Exact: every term a multiple of 2^emin (none truncated) and the
    // magnitudes summing below 2^(53 + emin) -- then the reference's
    // sequential sum and this one are the same exact value, a double.
    if (emin[q] == INT_MAX) exact_ok[q] = true;  // all terms zero
    else exact_ok[q] = emin[q] >= kFix && a[q] < ldexp(1.0, 53 + emin[q]);
  }
  bool ok = force_fallback == 0 && !ovf;
  for (int d = 0; d < 3 && ok; ++d) {
    float v;
    if (exact_ok[3] && exact_ok[d] && sd[3] != 0.0) {
      N.xc[d] = __double2float_rn(__ddiv_rn(sd[d], sd[3]));
      continue;
    }
    double bd[2];
    const int qs[2] = {d, 3};
    for (int t = 0; t < 2; ++t) {
      const int q = qs[t];
      const bool trunc = emin[q] != INT_MAX && emin[q] < kFix;
      bd[t] = g * a[q] + fabs(sd[q]) * 0x1p-52 + (trunc ? n * ldexp(1.0, kFix) : 0.0);
    }
    if (certify(sd[d], bd[0], sd[3], bd[1], &v)) N.xc[d] = v;
    else ok = false;
  }
  return ok;
}

__device__ void finish_node(DNode &N, int32_t node, const __int128 *s, double *a, const float *lo,
                            const float *hi, const int *emin, bool ovf, int32_t *fallback,
                            int64_t *counters, int32_t force_fallback, int32_t nd) {
  if (!decide_node(N, s, a, lo, hi, emin, ovf, force_fallback, nd)) {
    const unsigned long long k = atomicAdd((unsigned long long *)&counters[C_NFALLBACK], 1ull);
    fallback[k] = node;
  }
}

__device__ __forceinline__ void read_part(const double *p, __int128 *s, double *a, float *lo,
                                          float *hi, int *emin, int &ovf) {
  const __int128 *ps = reinterpret_cast<const __int128 *>(p);
  const float *pb = reinterpret_cast<const float *>(p + 12);
  const int *pe = reinterpret_cast<const int *>(p + 15);
  for (int q = 0; q < 4; ++q) {
    s[q] += ps[q];
    a[q] += p[8 + q];
    emin[q] = min(emin[q], pe[q]);
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = fminf(lo[d], pb[d]);
    hi[d] = fmaxf(hi[d], pb[3 + d]);
  }
  ovf |= pe[4];
}

// One warp per node of more than one chunk: reduce the chunk partials and
// finish the node.
__global__ void k_stats_final(DNode *nodes, int32_t nb, int32_t ne, const int64_t *chunk_base,
                              const double *part, int32_t *fallback, int64_t *counters,
                              int32_t force_fallback, int32_t nd, bool all) {
  const int32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int32_t node = nb + wid;
  if (node >= ne) return;
  DNode &N = nodes[node];
  const int64_t nc = (int64_t(N.count) + kChunk - 1) / kChunk;
  if (N.count <= 0 || (nc <= 1 && !all)) return;  // k_stats_final_one (unless `all`)
  const int64_t cb = chunk_base[wid];
  __int128 s[4] = {0, 0, 0, 0};
  double a[4] = {0, 0, 0, 0};
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  int emin[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
  int ovf = 0;
  for (int64_t c = lane; c < nc; c += 32) read_part(part + (cb + c) * kPartWords, s, a, lo, hi, emin, ovf);
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) s[q] += shfl_xor_i128(s[q], o);
    a[q] = warp_sum(a[q]);
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = warp_min(lo[d]);
    hi[d] = warp_max(hi[d]);
  }
  for (int q = 0; q < 4; ++q)
    for (int o = 16; o > 0; o >>= 1) emin[q] = min(emin[q], __shfl_xor_sync(0xffffffffu, emin[q], o));
  ovf = __any_sync(0xffffffffu, ovf != 0);
  if (lane != 0) return;
  finish_node(N, node, s, a, lo, hi, emin, ovf != 0, fallback, counters, force_fallback, nd);
}

// One block per node, for the top levels (nodes of many chunks): the warps
// reduce strided chunk subsets, thread 0 the warps' results, then finishes.
__global__ void __launch_bounds__(256)
    k_stats_final_block(DNode *nodes, int32_t nb, int32_t ne, const int64_t *chunk_base,
                        const double *part, int32_t *fallback, int64_t *counters,
                        int32_t force_fallback, int32_t nd) {
  const int32_t node = nb + int32_t(blockIdx.x);
  if (node >= ne) return;
  DNode &N = nodes[node];
  if (N.count <= 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nc = (int64_t(N.count) + kChunk - 1) / kChunk;
  const int64_t cb = chunk_base[blockIdx.x];
  __int128 s[4] = {0, 0, 0, 0};
  double a[4] = {0, 0, 0, 0};
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  int emin[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
  int ovf = 0;
  for (int64_t c = threadIdx.x; c < nc; c += 256)
    read_part(part + (cb + c) * kPartWords, s, a, lo, hi, emin, ovf);
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) s[q] += shfl_xor_i128(s[q], o);
    a[q] = warp_sum(a[q]);
    for (int o = 16; o > 0; o >>= 1) emin[q] = min(emin[q], __shfl_xor_sync(0xffffffffu, emin[q], o));
  }
  for (int d = 0; d < 3; ++d) {
    lo[d] = warp_min(lo[d]);
    hi[d] = warp_max(hi[d]);
  }
  ovf = __any_sync(0xffffffffu, ovf != 0);
  __shared__ __int128 ws[8][4];
  __shared__ double wa[8][4];
  __shared__ float wb[8][6];
  __shared__ int we[8][5];
  if (lane == 0) {
    for (int q = 0; q < 4; ++q) {
      ws[warp][q] = s[q];
      wa[warp][q] = a[q];
      we[warp][q] = emin[q];
    }
    for (int d = 0; d < 3; ++d) {
      wb[warp][d] = lo[d];
      wb[warp][3 + d] = hi[d];
    }
    we[warp][4] = ovf;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < 8; ++w) {
    for (int q = 0; q < 4; ++q) {
      s[q] += ws[w][q];
      a[q] += wa[w][q];
      emin[q] = min(emin[q], we[w][q]);
    }
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], wb[w][d]);
      hi[d] = fmaxf(hi[d], wb[w][3 + d]);
    }
    ovf |= we[w][4];
  }
  finish_node(N, node, s, a, lo, hi, emin, ovf != 0, fallback, counters, force_fallback, nd);
}

// One thread per node of a single chunk (most nodes of the deep levels): the
// per-node arithmetic, much of it FP64, then fills whole warps.
__global__ void k_stats_final_one(DNode *nodes, int32_t nb, int32_t ne, const int64_t *chunk_base,
                                  const double *part, int32_t *fallback, int64_t *counters,
                                  int32_t force_fallback, int32_t nd) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t node = nb + i;
  if (node >= ne) return;
  DNode &N = nodes[node];
  if (N.count <= 0 || N.count > kChunk) return;
  __int128 s[4] = {0, 0, 0, 0};
  double a[4] = {0, 0, 0, 0};
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  int emin[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
  int ovf = 0;
  read_part(part + chunk_base[i] * kPartWords, s, a, lo, hi, emin, ovf);
  finish_node(N, node, s, a, lo, hi, emin, ovf != 0, fallback, counters, force_fallback, nd);
}

// ---------------------------------------------------------------------------
// Tight certification of the centre of mass for the nodes the loose bound
// could not decide (k_stats_final's fallback list, at most kTightNodes of
// them per level).  The reference's sequential sum s_k = fl(s_{k-1} + t_k)
// differs from the exact sum by sum_k d_k, where the rounding error d_k is
// zero when s_{k-1} and t_k are both multiples of ulp(s_k) (then the exact
// sum is representable), and |d_k| <= ulp(s_k) / 2 otherwise.  ulp(s_k) is
// bounded from the exact prefix sums P_k: |s_k - P_k| is below the loose
// bound, so the binade of s_k lies within that of [P_k - E, P_k + E].  The
// resulting bound B counts only the terms that can round, which for
// coordinates of O(100) is a few thousand times ulp, not n ulp: the quotient
// is then decided on both sides of the bound far more often.  The exact sum
// itself is taken in double-double (error far below B).  Nodes the tight
// bound cannot decide either stay on the list for the sequential sum.
// ---------------------------------------------------------------------------
constexpr int kTightChunk = 2048;   // elements per chunk (8 per thread)
constexpr int kTightThreads = 256;
constexpr int kTightNodes = 64;     // fallback nodes per level taken by this pass
// blocks of the tight-certification passes: two per SM (grid-stride over chunks)
inline unsigned tight_blocks() { return unsigned(2 * sm_count()); }

struct TightChunk {  // per chunk of a listed node
  double hi[4], lo[4];  // double-double sum of the chunk's terms (x, y, z, m)
  double a[4];          // sum of |terms|
  double pre[4];        // approximate prefix sum of the terms before the chunk
};
struct TightNode {
  double hi[4], lo[4], a[4];
  double b[4];          // rounding-error bound of the sequential sum
};

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
__device__ __forceinline__ void dd_add(double &hi, double &lo, double bhi, double blo) {
  double s, e;
  two_sum(hi, bhi, s, e);
  e = __dadd_rn(e, __dadd_rn(lo, blo));
  hi = __dadd_rn(s, e);
  lo = __dsub_rn(e, __dsub_rn(hi, s));
}

// Chunks of the listed nodes in one index space: node f owns chunks
// [cbase[f], cbase[f + 1]).  Computed per block into shared memory.
__device__ int tight_layout(const DNode *nodes, const int32_t *fallback, const int64_t *counters,
                            int32_t *cbase, int32_t skip) {
  const int nt = skip ? 0 : int(min64(counters[C_NFALLBACK], kTightNodes));
  if (threadIdx.x == 0) {
    int32_t run = 0;
    for (int f = 0; f < nt; ++f) {
      cbase[f] = run;
      run += (nodes[fallback[f]].count + kTightChunk - 1) / kTightChunk;
    }
    cbase[nt] = run;
  }
  __syncthreads();
  return nt;
}

__device__ __forceinline__ void terms_of(const float4 &p, double t[4], int lsb[4]) {
  const float fx = fmul_(p.w, p.x), fy = fmul_(p.w, p.y), fz = fmul_(p.w, p.z);
  t[0] = double(fx);
  t[1] = double(fy);
  t[2] = double(fz);
  t[3] = double(p.w);
  lsb[0] = lsb_exp(fx);
  lsb[1] = lsb_exp(fy);
  lsb[2] = lsb_exp(fz);
  lsb[3] = lsb_exp(p.w);
}

// Pass 1: double-double chunk sums; the last block to finish forms each
// node's chunk prefixes and totals.
__global__ void __launch_bounds__(kTightThreads)
    k_cm_tight_sums(const float4 *__restrict__ pos, const DNode *nodes, const int32_t *fallback,
                    int64_t *counters, TightChunk *chunks, TightNode *tn, int32_t skip) {
  __shared__ int32_t cbase[kTightNodes + 1];
  __shared__ double red[kTightThreads / 32][12];
  __shared__ int last;
  const int nt = tight_layout(nodes, fallback, counters, cbase, skip);
  const int total = cbase[nt];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int f = 0;
    while (f + 1 < nt && cbase[f + 1] <= g) ++f;
    const DNode &N = nodes[fallback[f]];
    const int64_t b0 = int64_t(N.offset) + int64_t(g - cbase[f]) * kTightChunk;
    const int64_t e0 = min64(int64_t(N.offset) + N.count, b0 + kTightChunk);
    double hi[4] = {0, 0, 0, 0}, lo[4] = {0, 0, 0, 0}, a[4] = {0, 0, 0, 0};
    for (int64_t i = b0 + threadIdx.x; i < e0; i += kTightThreads) {
      double t[4];
      int lsb[4];
      terms_of(pos[i], t, lsb);
      for (int q = 0; q < 4; ++q) {
        dd_add(hi[q], lo[q], t[q], 0.0);
        a[q] = __dadd_ru(a[q], fabs(t[q]));
      }
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int q = 0; q < 4; ++q) {
        const double oh = __shfl_xor_sync(0xffffffffu, hi[q], o);
        const double ol = __shfl_xor_sync(0xffffffffu, lo[q], o);
        dd_add(hi[q], lo[q], oh, ol);
        a[q] = __dadd_ru(a[q], __shfl_xor_sync(0xffffffffu, a[q], o));
      }
    if (lane == 0)
      for (int q = 0; q < 4; ++q) {
        red[warp][q] = hi[q];
        red[warp][4 + q] = lo[q];
        red[warp][8 + q] = a[q];
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      TightChunk c{};
      for (int q = 0; q < 4; ++q) {
        c.hi[q] = red[0][q];
        c.lo[q] = red[0][4 + q];
        c.a[q] = red[0][8 + q];
      }
      for (int w = 1; w < kTightThreads / 32; ++w)
        for (int q = 0; q < 4; ++q) {
          dd_add(c.hi[q], c.lo[q], red[w][q], red[w][4 + q]);
          c.a[q] = __dadd_ru(c.a[q], red[w][8 + q]);
        }
      chunks[g] = c;
    }
    __syncthreads();
  }
  // the last block to finish forms the prefixes and totals
  __threadfence();
  if (threadIdx.x == 0)
    last = atomicAdd((unsigned long long *)&counters[C_TDONE1], 1ull) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int f = threadIdx.x; f < nt; f += blockDim.x) {
    double hi[4] = {0, 0, 0, 0}, lo[4] = {0, 0, 0, 0}, a[4] = {0, 0, 0, 0};
    for (int32_t g = cbase[f]; g < cbase[f + 1]; ++g) {
      TightChunk &c = chunks[g];
      for (int q = 0; q < 4; ++q) {
        c.pre[q] = hi[q] + lo[q];
        dd_add(hi[q], lo[q], c.hi[q], c.lo[q]);
        a[q] = __dadd_ru(a[q], c.a[q]);
      }
    }
    for (int q = 0; q < 4; ++q) {
      tn[f].hi[q] = hi[q];
      tn[f].lo[q] = lo[q];
      tn[f].a[q] = a[q];
      tn[f].b[q] = 0.0;
    }
  }
  if (threadIdx.x == 0) counters[C_TDONE1] = 0;
}

// Binade exponent range of the values in [v - e, v + e].
__device__ __forceinline__ void binades(double v, double e, int &emin, int &emax) {
  const double lo = v - e, hi = v + e;
  const double amax = fmax(fabs(lo), fabs(hi));
  emax = amax > 0.0 ? ilogb(amax) : -1074;
  if (lo <= 0.0 && hi >= 0.0) emin = -1074;
  else emin = ilogb(fmin(fabs(lo), fabs(hi)));
}

// Pass 2: the rounding-error bound per listed node; the last block certifies
// and writes the centres of mass (certified nodes leave the list as -1).
__global__ void __launch_bounds__(kTightThreads)
    k_cm_tight_bound(const float4 *__restrict__ pos, DNode *nodes, int32_t *fallback,
                     int64_t *counters, const TightChunk *chunks, TightNode *tn, int32_t skip) {
  __shared__ int32_t cbase[kTightNodes + 1];
  __shared__ float4 el[kTightChunk];
  __shared__ double wsum[kTightThreads / 32][4];
  __shared__ double bred[kTightThreads / 32][4];
  __shared__ int last;
  const int nt = tight_layout(nodes, fallback, counters, cbase, skip);
  const int total = cbase[nt];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kPerT = kTightChunk / kTightThreads;
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int f = 0;
    while (f + 1 < nt && cbase[f + 1] <= g) ++f;
    const DNode &N = nodes[fallback[f]];
    const int64_t b0 = int64_t(N.offset) + int64_t(g - cbase[f]) * kTightChunk;
    const int len = int(min64(int64_t(N.offset) + N.count - b0, kTightChunk));
    for (int i = threadIdx.x; i < len; i += kTightThreads) el[i] = pos[b0 + i];
    __syncthreads();
    // this thread's elements [8 tid, 8 tid + 8): local sums, then a block scan
    double loc[4] = {0, 0, 0, 0};
    for (int k = 0; k < kPerT; ++k) {
      const int i = threadIdx.x * kPerT + k;
      if (i < len) {
        double t[4];
        int lsb[4];
        terms_of(el[i], t, lsb);
        for (int q = 0; q < 4; ++q) loc[q] += t[q];
      }
    }
    double inc[4];
    for (int q = 0; q < 4; ++q) {
      inc[q] = loc[q];
      for (int o = 1; o < 32; o <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, inc[q], o);
        if (lane >= o) inc[q] += v;
      }
      if (lane == 31) wsum[warp][q] = inc[q];
    }
    __syncthreads();
    const TightChunk &C = chunks[g];
    const TightNode &T = tn[f];
    double P[4], E[4], bsum[4] = {0, 0, 0, 0};
    for (int q = 0; q < 4; ++q) {
      double wpre = 0;
      for (int w = 0; w < warp; ++w) wpre += wsum[w][q];
      P[q] = C.pre[q] + wpre + (inc[q] - loc[q]);
      // |s_k - P_k| (sequential error) and the error of this approximate
      // prefix are each below (n + 64) u sum|t|
      E[q] = 4.0 * (double(N.count) + 64.0) * 0x1p-53 * T.a[q];
    }
    for (int k = 0; k < kPerT; ++k) {
      const int i = threadIdx.x * kPerT + k;
      if (i >= len) break;
      double t[4];
      int lsb[4];
      terms_of(el[i], t, lsb);
      const bool first = b0 + i == N.offset;
      for (int q = 0; q < 4; ++q) {
        const double prev = P[q];
        P[q] += t[q];
        if (first || t[q] == 0.0) continue;  // 0 + t and s + 0 are exact
        int pmin, pmax, cmin, cmax;
        binades(prev, E[q], pmin, pmax);
        binades(P[q], E[q], cmin, cmax);
        const int ulp_e = max(cmax, -1022) - 52;  // largest possible ulp(s_k)
        const bool exact = pmin >= cmax && lsb[q] != INT_MIN && lsb[q] >= ulp_e;
        if (!exact) bsum[q] = __dadd_ru(bsum[q], ldexp(1.0, ulp_e - 1));
      }
    }
    for (int q = 0; q < 4; ++q) {
      for (int o = 16; o > 0; o >>= 1) bsum[q] = __dadd_ru(bsum[q], __shfl_xor_sync(0xffffffffu, bsum[q], o));
      if (lane == 0) bred[warp][q] = bsum[q];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int q = 0; q < 4; ++q) {
        double b = 0;
        for (int w = 0; w < kTightThreads / 32; ++w) b = __dadd_ru(b, bred[w][q]);
        if (b > 0) atomicAdd(&tn[f].b[q], b);
      }
    __syncthreads();
  }
  __threadfence();
  if (threadIdx.x == 0)
    last = atomicAdd((unsigned long long *)&counters[C_TDONE2], 1ull) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int f = threadIdx.x; f < nt; f += blockDim.x) {
    const TightNode &T = tn[f];
    DNode &N = nodes[fallback[f]];
    double sx[4], bx[4];
    for (int q = 0; q < 4; ++q) {
      sx[q] = T.hi[q] + T.lo[q];
      // B (atomics rounded to nearest: slack), the double-double error and
      // the rounding of hi + lo
      bx[q] = T.b[q] * (1.0 + 0x1p-30) + (double(N.count) + 64.0) * 0x1p-98 * T.a[q] +
              fabs(sx[q]) * 0x1p-52;
    }
    float v[3];
    bool ok = true;
    for (int d = 0; d < 3 && ok; ++d) ok = certify(sx[d], bx[d], sx[3], bx[3], &v[d]);
    if (ok) {
      for (int d = 0; d < 3; ++d) N.xc[d] = v[d];
      fallback[f] = -1;
      atomicAdd((unsigned long long *)&counters[C_NTIGHT], 1ull);
    }
  }
  if (threadIdx.x == 0) counters[C_TDONE2] = 0;
}

// The reference's centre of mass for the listed nodes, summed sequentially
// in array order in double (BGQCM.c:186-211).
__global__ void k_cm_fallback(const float4 *__restrict__ pos, DNode *nodes, const int32_t *fallback,
                              const int64_t *counters) {
  const int64_t nf = counters[C_NFALLBACK];
  for (int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; f < nf;
       f += int64_t(gridDim.x) * blockDim.x) {
    if (fallback[f] < 0) continue;  // certified by the tight pass
    DNode &N = nodes[fallback[f]];
    double x = 0, y = 0, z = 0, m = 0;
    for (int32_t i = 0; i < N.count; ++i) {
      const float4 p = pos[N.offset + i];
      x = __dadd_rn(x, double(fmul_(p.w, p.x)));
      y = __dadd_rn(y, double(fmul_(p.w, p.y)));
      z = __dadd_rn(z, double(fmul_(p.w, p.z)));
      m = __dadd_rn(m, double(p.w));
    }
    N.xc[0] = __double2float_rn(__ddiv_rn(x, m));
    N.xc[1] = __double2float_rn(__ddiv_rn(y, m));
    N.xc[2] = __double2float_rn(__ddiv_rn(z, m));
  }
}

__device__ __forceinline__ float key_of(const float4 &p, int d) {
  return d == 0 ? p.x : (d == 1 ? p.y : p.z);
}

// Block-wide exclusive scan of one int per thread.
__device__ __forceinline__ int block_excl_scan(int v, int *sh_warp, int *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? sh_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    sh_warp[lane] = w;
  }
  __syncthreads();
  const int excl = x - v + (warp > 0 ? sh_warp[warp - 1] : 0);
  *total = sh_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return excl;
}

// Left counts of each chunk of a splitting node; in block mode also each
// warp's left elements before its share of the chunk (the shares of
// k_part_left: warp w takes [w * kChunk / 8, (w + 1) * kChunk / 8)).  Only
// the split coordinate is loaded, every lane's loads in flight at once.
template <bool WM>
__global__ void __launch_bounds__(kChunkThreads)
    k_part_count(const float4 *__restrict__ pos, const DNode *nodes, const int32_t *chunk_node,
                 const int64_t *chunk_base, int32_t nb, const int64_t *nchunk, int32_t *left_cnt,
                 int32_t *wpre) {
  CHUNK_PROLOGUE
  const ChunkRange R = chunk_range(nodes, chunk_node, chunk_base, nb, chunk);
  const DNode &N = nodes[R.node];
  if (N.split_dim < 0) {
    if (tid == 0) left_cnt[chunk] = 0;
    return;
  }
  const int d = N.split_dim;
  const float split = N.xc[d];
  const float *key = reinterpret_cast<const float *>(pos + R.begin) + d;
  if (WM) {
    int c = 0;
    for (int k = tid; k < R.len; k += NT) c += key[4 * k] < split;
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane_ == 0) left_cnt[chunk] = c;
    return;
  }
  constexpr int kWarps = kChunkThreads / 32, kSub = kChunk / kWarps, kPer = kSub / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float kv[kPer];
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const int e = warp * kSub + 32 * u + lane;
    kv[u] = e < R.len ? key[4 * e] : INFINITY;
  }
  int c = 0;
#pragma unroll
  for (int u = 0; u < kPer; ++u) c += kv[u] < split;
  c = __reduce_add_sync(0xffffffffu, c);
  __shared__ int wt[kWarps];
  if (lane == 0) wt[warp] = c;
  __syncthreads();
  if (threadIdx.x < kWarps) {
    int pre = 0, tot = 0;
    for (int w = 0; w < kWarps; ++w) {
      pre += w < int(threadIdx.x) ? wt[w] : 0;
      tot += wt[w];
    }
    wpre[chunk * kWarps + threadIdx.x] = pre;
    if (threadIdx.x == 0) left_cnt[chunk] = tot;
  }
}

// Per splitting node, a warp each: exclusive scan of its chunks' left counts
// (in chunk order) and the node's total.
__global__ void k_part_node_scan(DNode *nodes, int32_t nb, int32_t ne, const int64_t *chunk_base,
                                 const int32_t *left_cnt, int64_t *left_base) {
  const int32_t w = int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (nb + w >= ne) return;  // whole warps
  DNode &N = nodes[nb + w];
  if (N.split_dim < 0) return;
  const int64_t cb = chunk_base[w];
  const int64_t nc = (int64_t(N.count) + kChunk - 1) / kChunk;
  int64_t run = 0;
  for (int64_t c0 = 0; c0 < nc; c0 += 32) {
    const int64_t c = c0 + lane;
    const int64_t v = c < nc ? left_cnt[cb + c] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (c < nc) left_base[cb + c] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) N.nleft = int32_t(run);
}

// Left particles go to their rank; idx[rank] records where each came from.
// Warp w takes the chunk's elements [w * kSub, (w + 1) * kSub) 32 at a time
// (coalesced), kB steps' loads in flight; ranks follow array order through
// the warps' left counts before them (k_part_count) and a ballot prefix
// within each step.
template <bool WM>
__global__ void __launch_bounds__(kChunkThreads)
    k_part_left(const float4 *__restrict__ pos, const int32_t *__restrict__ oid, const DNode *nodes,
                const int32_t *chunk_node, const int64_t *chunk_base, int32_t nb,
                const int64_t *nchunk, const int64_t *left_base, const int32_t *wpre, float4 *tpos,
                int32_t *toid, int32_t *idx, int32_t *ridx) {
  constexpr int kWarps = kChunkThreads / 32;
  constexpr int kSub = WM ? kChunk : kChunk / kWarps;  // a warp's share of the chunk
  constexpr int kB = 4;
  CHUNK_PROLOGUE
  const ChunkRange R = chunk_range(nodes, chunk_node, chunk_base, nb, chunk);
  const DNode &N = nodes[R.node];
  if (N.split_dim < 0) {
    // a leaf keeps its elements: copied once into the next level's buffer
    for (int k = tid; k < R.len; k += NT) {
      tpos[R.begin + k] = pos[R.begin + k];
      toid[R.begin + k] = oid[R.begin + k];
    }
    return;
  }
  const int d = N.split_dim;
  const float split = N.xc[d];
  const int32_t off = N.offset, nleft = N.nleft;
  const int lane = threadIdx.x & 31, warp = WM ? 0 : int(threadIdx.x >> 5);
  const unsigned below = (1u << lane) - 1u;
  const int sub_end = min(kSub, R.len - warp * kSub);  // elements of this warp's share
  int r = int(left_base[chunk]) + (WM ? 0 : wpre[chunk * kWarps + warp]);
  for (int j0 = 0; j0 < sub_end; j0 += 32 * kB) {
    float4 p[kB];
    int32_t o[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const int e = warp * kSub + j0 + 32 * u + lane;
      if (j0 + 32 * u < sub_end && e < R.len) {
        p[u] = pos[R.begin + e];
        o[u] = oid[R.begin + e];
      } else {
        p[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        o[u] = 0;
      }
    }
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      if (j0 + 32 * u >= sub_end) break;  // the same for the whole warp
      const int e = warp * kSub + j0 + 32 * u + lane;
      const bool in = e < R.len;
      const bool l = in && key_of(p[u], d) < split;
      const unsigned bal = __ballot_sync(0xffffffffu, l);
      const int q = r + __popc(bal & below);  // left elements before this one
      if (l) {
        tpos[off + q] = p[u];
        toid[off + q] = o[u];
        idx[off + q] = R.local + e;
      } else if (in) {
        ridx[off + (R.local + e - q)] = R.local + e;
        if (R.local + e >= nleft) {
          // a right element at or after nleft: no swap touches it, it stays
          tpos[R.begin + e] = p[u];
          toid[R.begin + e] = o[u];
        }
      }
      r += __popc(bal);
    }
  }
}

// A swap chain still running after the partition's single steps: its
// position in the node, the node and the element's position in the level's
// array.
struct ChainItem {
  int32_t q, node;
  int64_t src;
};
static_assert(sizeof(ChainItem) == sizeof(int4), "a chain item fills one int4 of the queue");

// One or more steps of the chain q -> idx[q] -> ... (q < nleft): the q-th
// left element has c = idx[q] - q right elements before it, and so has every
// left element up to the c-th right element (at ridx[c]), whose ranks run to
// b = ridx[c] - c.  Within that run each step adds c, so the chain leaves
// [q, min(b, nleft)) at the first of q + c, q + 2c, ... at or past it.
// Returns a position > q; *bad on an inconsistent partition.
__device__ __forceinline__ int32_t chain_jump(int32_t q, int32_t nleft, int32_t nright,
                                              const int32_t *idx, const int32_t *ridx, bool *bad) {
  const int32_t c = idx[q] - q;
  if (c <= 0) {  // cannot happen for a valid partition (a chain never meets a fixed point)
    *bad = true;
    return nleft;
  }
  int32_t lim = nleft;
  if (c < nright) {
    const int32_t b = ridx[c] - c;
    if (b <= q) {  // cannot happen for a valid partition
      *bad = true;
      return nleft;
    }
    lim = min(lim, b);
  }
  const int32_t k = lim > q + c ? (lim - q + c - 1) / c : 1;
  return q + k * c;
}

// The other particles: those at or after position nleft stay (k_part_left
// writes them); one at p < nleft moves along p -> idx[p] -> ... until it
// lands at or after nleft (the reference's swap sequence,
// RCBForceTree.cxx:647-669), taken a run of equal steps at a time
// (chain_jump).  Positions increase strictly along a chain, so it ends within
// count jumps.
template <bool WM>
__global__ void __launch_bounds__(kChunkThreads)
    k_part_right(const float4 *__restrict__ pos, const int32_t *__restrict__ oid, const DNode *nodes,
                 const int32_t *chunk_node, const int64_t *chunk_base, int32_t nb,
                 const int64_t *nchunk, const int32_t *__restrict__ idx,
                 const int32_t *__restrict__ ridx, float4 *tpos, int32_t *toid, int32_t *err,
                 int64_t *counters, ChainItem *chains, int64_t chain_cap) {
  CHUNK_PROLOGUE
  const ChunkRange R = chunk_range(nodes, chunk_node, chunk_base, nb, chunk);
  const DNode &N = nodes[R.node];
  if (N.split_dim < 0) return;
  const int d = N.split_dim;
  const float split = N.xc[d];
  const int32_t is = N.nleft, nright = N.count - N.nleft;
  const int32_t *nidx = idx + N.offset, *nridx = ridx + N.offset;
  if (R.local >= is) return;  // every element here stays (k_part_left)
  if (WM) {
    for (int k = tid; k < R.len && R.local + k < is; k += NT) {
      const int64_t src = R.begin + k;
      const float4 p = pos[src];
      if (key_of(p, d) < split) continue;
      int32_t q = R.local + k;
      int32_t steps = 0;
      bool bad = false;
      while (q < is && steps <= N.count && !bad) {
        if (steps++ < kPlainSteps) {  // single steps first: most chains end within a few
          const int32_t nq = nidx[q];
          if (nq <= q) bad = true;
          q = nq;
        } else {
          q = chain_jump(q, is, nright, nidx, nridx, &bad);
        }
      }
      if (q < is || bad || q >= N.count) {
        atomicExch(err, 2);
        continue;
      }
      tpos[N.offset + q] = p;
      toid[N.offset + q] = oid[src];
    }
    return;
  }
  // Block mode: the thread's 16 elements take their first kPlainSteps steps
  // in lockstep, so up to 16 independent loads are in flight per step (most
  // chains end within a few).  The chains still running go to the level's
  // chain queue (k_part_chains follows them a chain per thread): long chains
  // gather in a few regions of a level, thousands in one chunk.
  constexpr int kPerT = kChunk / kChunkThreads;
  const float *key = reinterpret_cast<const float *>(pos + R.begin) + d;
  int32_t q[kPerT];
  unsigned right = 0;
#pragma unroll
  for (int j = 0; j < kPerT; ++j) {
    const int k = tid + j * NT;
    q[j] = R.local + k;
    if (k < R.len && q[j] < is && !(key[4 * k] < split)) right |= 1u << j;
  }
  unsigned active = right;
  bool bad = false;
  for (int32_t step = 0; active && step < kPlainSteps; ++step) {
    int32_t nq[kPerT];
#pragma unroll
    for (int j = 0; j < kPerT; ++j) nq[j] = (active >> j & 1u) ? nidx[q[j]] : q[j];
#pragma unroll
    for (int j = 0; j < kPerT; ++j) {
      if (!(active >> j & 1u)) continue;
      if (nq[j] <= q[j] || nq[j] >= N.count) {  // cannot happen for a valid partition
        bad = true;
        active &= ~(1u << j);
        right &= ~(1u << j);
        continue;
      }
      q[j] = nq[j];
      if (nq[j] >= is) active &= ~(1u << j);
    }
  }
  // one queue reservation per warp
  const int lane = threadIdx.x & 31;
  const int na = __popc(active);
  int incl = na;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  unsigned long long base = 0;
  if (lane == 31 && incl > 0)
    base = atomicAdd((unsigned long long *)&counters[C_CHAINS], (unsigned long long)incl);
  base = __shfl_sync(0xffffffffu, base, 31);
  int64_t slot = int64_t(base) + incl - na;
#pragma unroll
  for (int j = 0; j < kPerT; ++j) {
    if (!(right >> j & 1u)) continue;
    const int64_t src = R.begin + tid + j * NT;
    if (active >> j & 1u) {
      if (slot < chain_cap) chains[slot] = ChainItem{q[j], R.node, src};
      else bad = true;  // cannot happen: a chain per element at most
      ++slot;
      continue;
    }
    tpos[N.offset + q[j]] = pos[src];
    toid[N.offset + q[j]] = oid[src];
  }
  if (bad) atomicExch(err, 2);
}

// The level's long swap chains, a thread each, a run of equal steps at a
// time (chain_jump); each lands its element.
__global__ void __launch_bounds__(256)
    k_part_chains(const float4 *__restrict__ pos, const int32_t *__restrict__ oid,
                  const DNode *nodes, const ChainItem *__restrict__ chains, int64_t chain_cap,
                  const int64_t *counters, const int32_t *__restrict__ idx,
                  const int32_t *__restrict__ ridx, float4 *tpos, int32_t *toid, int32_t *err) {
  const int64_t nq = min64(counters[C_CHAINS], chain_cap);
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < nq;
       c += int64_t(gridDim.x) * blockDim.x) {
    const ChainItem it = chains[c];
    const DNode &N = nodes[it.node];
    const int32_t is = N.nleft, nright = N.count - N.nleft;
    const int32_t *nidx = idx + N.offset, *nridx = ridx + N.offset;
    int32_t qq = it.q;
    bool b = false;
    for (int32_t k = 0; qq < is && k <= N.count && !b; ++k)
      qq = chain_jump(qq, is, nright, nidx, nridx, &b);
    if (b || qq < is || qq >= N.count) {  // cannot happen for a valid partition
      atomicExch(err, 2);
      continue;
    }
    tpos[N.offset + qq] = pos[it.src];
    toid[N.offset + qq] = oid[it.src];
  }
}

// The whole partition of one node in one block, for levels whose nodes hold
// at most kNodeMax elements: the left elements go to their ranks (warp w
// takes a contiguous share of the node, ranks in array order through the
// warps' totals and ballot prefixes), their source positions into shared
// memory, and every right element before nleft follows p -> idx[p] -> ...
// there (the reference's swap sequence, RCBForceTree.cxx:647-669).  A chain
// longer than kChainSteps sends the block to pointer jumping in place over
// idx (each entry moves along its own chain, so every read sees a point of
// that chain), which ends in log2(count) + 1 rounds.  Also sets N.nleft and
// copies leaves' elements.
template <int NT>
__global__ void __launch_bounds__(NT)
    k_part_node(const float4 *__restrict__ pos, const int32_t *__restrict__ oid, DNode *nodes,
                int32_t nb, int32_t ne, int32_t node_max, float4 *tpos, int32_t *toid,
                int32_t *err) {
  extern __shared__ int32_t sidx[];
  constexpr int kW = NT / 32;
  __shared__ int wtot[kW];
  __shared__ int s_long;
  const int32_t node = nb + int32_t(blockIdx.x);
  if (node >= ne) return;
  DNode &N = nodes[node];
  const int cnt = N.count;
  if (cnt > node_max) {  // the launch's shared memory does not hold it
    if (threadIdx.x == 0) atomicExch(err, 3);
    return;
  }
  const int64_t off = N.offset;
  if (N.split_dim < 0) {
    for (int e = threadIdx.x; e < cnt; e += NT) {
      tpos[off + e] = pos[off + e];
      toid[off + e] = oid[off + e];
    }
    return;
  }
  const int d = N.split_dim;
  const float split = N.xc[d];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  const int sub = (((cnt + kW - 1) / kW) + 31) & ~31;
  const int beg = warp * sub, end = min(cnt, beg + sub);
  if (threadIdx.x == 0) s_long = 0;
  // four loads in flight per lane in both passes
  constexpr int kU = 4;
  int c = 0;
  for (int e0 = beg; e0 < end; e0 += 32 * kU) {
    float key[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + 32 * u + lane;
      key[u] = e < end ? key_of(pos[off + e], d) : split;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) c += __popc(__ballot_sync(0xffffffffu, key[u] < split));
  }
  if (lane == 0) wtot[warp] = c;
  __syncthreads();
  int r = 0, nleft = 0;
#pragma unroll
  for (int w = 0; w < kW; ++w) {
    const int v = wtot[w];
    r += w < warp ? v : 0;
    nleft += v;
  }
  for (int e0 = beg; e0 < end; e0 += 32 * kU) {
    float4 pu[kU];
    int ou[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + 32 * u + lane;
      pu[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      ou[u] = 0;
      if (e < end) {
        pu[u] = pos[off + e];
        ou[u] = oid[off + e];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + 32 * u + lane;
      const bool l = e < end && key_of(pu[u], d) < split;
      const unsigned bal = __ballot_sync(0xffffffffu, l);
      if (l) {
        const int q = r + __popc(bal & below);
        tpos[off + q] = pu[u];
        toid[off + q] = ou[u];
        sidx[q] = e;
      } else if (e < end && e >= nleft) {
        // a right element at or after nleft: no swap touches it, it stays
        tpos[off + e] = pu[u];
        toid[off + e] = ou[u];
      }
      r += __popc(bal);
    }
  }
  if (threadIdx.x == 0) N.nleft = nleft;
  __syncthreads();
  for (int e = threadIdx.x; e < nleft; e += NT) {
    const float4 p = pos[off + e];
    if (key_of(p, d) < split) continue;
    int q = e, steps = 0;
    bool bad = false;
    while (q < nleft && steps < kChainSteps) {
      const int nq = sidx[q];
      if (nq <= q || nq >= cnt) {  // cannot happen for a valid partition
        bad = true;
        break;
      }
      q = nq;
      ++steps;
    }
    if (bad) {
      atomicExch(err, 2);
      continue;
    }
    if (q < nleft) {
      s_long = 1;
      continue;
    }
    tpos[off + q] = p;
    toid[off + q] = oid[off + e];
  }
  __syncthreads();
  if (!s_long) return;
  // pointer jumping: afterwards idx[q] is the end of the chain through q
  for (int round = 0;; ++round) {
    bool ch = false;
    for (int q = threadIdx.x; q < nleft; q += NT) {
      const int j = sidx[q];
      if (j != q && j < nleft) {  // j == q: a left element that no swap moves
        sidx[q] = sidx[j];
        ch = true;
      }
    }
    if (!__syncthreads_or(ch)) break;
    if (round > 40) {  // cannot happen for a valid partition
      if (threadIdx.x == 0) atomicExch(err, 2);
      return;
    }
  }
  for (int e = threadIdx.x; e < nleft; e += NT) {
    const float4 p = pos[off + e];
    if (key_of(p, d) < split) continue;
    const int q = sidx[e];
    if (q < nleft || q >= cnt) {
      atomicExch(err, 2);
      continue;
    }
    tpos[off + q] = p;
    toid[off + q] = oid[off + e];
  }
}

// ---------------------------------------------------------------------------
// Whole subtrees in one block.  Once every node of a level holds at most
// kSubMax elements, one block per node builds that node's entire subtree:
// level by level inside the block, each node's statistics (box, exact
// fixed-point centre-of-mass sums and their certification, the reference's
// sequential sum where the bounds leave it open), the split decision, the
// partition at the centre of mass (left elements to their ranks, right
// elements along the swap chains kept in shared memory, pointer jumping for
// long chains -- the reference's swap sequence, RCBForceTree.cxx:623-672) and
// the children.  The level's nodes are shared out to teams of warps: a whole
// block for one node, down to a warp per node on deep levels.  Elements
// alternate between the two element buffers as in the level loop (a leaf's
// elements are copied into the other buffer once, so both end up holding
// every leaf).  The subtree's nodes go to a scratch region (2 x count
// records per root, at twice the root's element offset) in per-root
// breadth-first order; k_subtree_place later numbers all of them by level
// and offset, as the level loop would have.  One launch and no host
// synchronisation replace the deep levels' kernels.
// ---------------------------------------------------------------------------
constexpr int kSubMax = 16384;       // largest subtree root (elements)
constexpr int kSubThreads = 512;   // two blocks per SM
constexpr int kSubWarps = kSubThreads / 32;
constexpr int kSubDepth = 48;        // deepest level below a root; deeper: the level loop

struct SubWarpStats {
  __int128 s[4];
  double a[4];
  float lo[3], hi[3];
  int emin[4];
  int ovf;
};

// Barrier over the warps [w0, w0 + nw) of the block: named barrier 1 + team
// for teams of several warps (at most 8 teams), __syncwarp for one warp.
__device__ __forceinline__ void team_sync(int team, int nw) {
  if (nw == 1) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(team + 1), "r"(nw * 32) : "memory");
  }
}

__global__ void __launch_bounds__(kSubThreads, 2)
    k_subtree(const DNode *__restrict__ nodes, int32_t nb, int32_t ne, float4 *epos, int32_t *eoid,
              float4 *tpos, int32_t *toid, DNode *sub, SubWarpStats *sub_stats, int32_t *sub_first,
              int64_t *hist, int32_t force_fallback, int32_t nd, int64_t *counters) {
  extern __shared__ int32_t sidx[];  // chain table by element position in the subtree
  __shared__ SubWarpStats wst[kSubWarps];
  __shared__ int wtot[kSubWarps];
  __shared__ int tflag[kSubWarps];      // per team: a chain too long / pointer jumping changed
  __shared__ int first[kSubDepth + 2];  // first local node of each depth
  __shared__ int sh_warp[32];
  __shared__ int s_nsplit;
  const int32_t r = int32_t(blockIdx.x);
  const int32_t nroots = ne - nb;
  const DNode R = nodes[nb + r];
  const int rcnt = R.count;
  const int32_t roff = R.offset;
  DNode *loc = sub + 2 * int64_t(roff);  // this root's 2 x count records
  // the reduced statistics of the current level's nodes, by position in the
  // level (a level holds at most count nodes)
  SubWarpStats *lst = sub_stats + roff;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  if (rcnt > kSubMax) {  // the launch's shared memory does not hold it
    if (threadIdx.x == 0) atomicExch(reinterpret_cast<int32_t *>(counters + C_ERR), 3);
    return;
  }
  if (threadIdx.x == 0) {
    loc[0] = R;
    loc[0].cl = loc[0].cr = 0;
    first[0] = 0;
    first[1] = 1;
  }
  __syncthreads();
  const float4 *src = epos;
  const int32_t *soid = eoid;
  float4 *dst = tpos;
  int32_t *doid = toid;
  int f0 = 0, f1 = 1, depth = 0;
  int nfb = 0;  // sequential centre-of-mass sums (thread 0 of a team counts)
  while (f1 > f0) {
    const int F = f1 - f0;
    // teams: the whole block for one node, halving per doubling of the level
    // to a warp per node from 9 nodes on (at most 8 teams of several warps,
    // named barriers 1-8)
    int nw = 1;
    if (F <= 8) {
      int p2 = 1;
      while (p2 < F) p2 <<= 1;
      nw = kSubWarps / p2;
    }
    const int nteams = kSubWarps / nw;
    const int team = warp / nw, w0 = team * nw, wi = warp - w0;
    const int tl = wi * 32 + lane, TN = nw * 32;
    // ---- statistics: a team per node, reduced into the level's scratch ----
    for (int f = f0 + team; f < f1; f += nteams) {
      const DNode N = loc[f];
      const int c = N.count;
      const int64_t o = N.offset;
      FixAcc fx[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) fx[q].zero();
      float fa[4] = {0.f, 0.f, 0.f, 0.f};
      float bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
      bool ovf = false;
      bool trn[4] = {false, false, false, false};
      int it = 0;
      for (int e = tl; e < c; e += TN, ++it) {
        const float4 p = src[o + e];
        const float w = p.w;
        const float t[4] = {fmul_(w, p.x), fmul_(w, p.y), fmul_(w, p.z), w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          fx[q].add(t[q], ovf, trn[q]);
          fa[q] = __fadd_ru(fa[q], fabsf(t[q]));
        }
        bl[0] = fminf(bl[0], p.x); bh[0] = fmaxf(bh[0], p.x);
        bl[1] = fminf(bl[1], p.y); bh[1] = fmaxf(bh[1], p.y);
        bl[2] = fminf(bl[2], p.z); bh[2] = fmaxf(bh[2], p.z);
        if ((it + 1) % kFoldTerms == 0) {
#pragma unroll
          for (int q = 0; q < 4; ++q) fx[q].fold();
        }
      }
      __int128 sq[4];
      int lsb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        fx[q].fold();
        sq[q] = fx[q].sum();
        lsb[q] = __reduce_min_sync(0xffffffffu, fx[q].lsb);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        for (int sft = 16; sft > 0; sft >>= 1) {
          sq[q] += shfl_xor_i128(sq[q], sft);
          fa[q] = __fadd_ru(fa[q], __shfl_xor_sync(0xffffffffu, fa[q], sft));
        }
      }
      int em[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool tq = __any_sync(0xffffffffu, trn[q]);
        em[q] = tq ? kFix - 1 : (lsb[q] == INT_MAX ? INT_MAX : kFix + lsb[q]);
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        bl[d] = warp_min(bl[d]);
        bh[d] = warp_max(bh[d]);
      }
      const bool wovf = __any_sync(0xffffffffu, ovf);
      SubWarpStats &W = nw == 1 ? lst[f - f0] : wst[warp];
      if (lane == 0) {
        for (int q = 0; q < 4; ++q) {
          W.s[q] = sq[q];
          W.a[q] = double(fa[q]);
          W.emin[q] = em[q];
        }
        for (int d = 0; d < 3; ++d) {
          W.lo[d] = bl[d];
          W.hi[d] = bh[d];
        }
        W.ovf = wovf ? 1 : 0;
      }
      if (nw > 1) {
        team_sync(team, nw);
        if (tl == 0) {
          SubWarpStats T = wst[w0];
          for (int w = 1; w < nw; ++w) {
            const SubWarpStats &V = wst[w0 + w];
            for (int q = 0; q < 4; ++q) {
              T.s[q] += V.s[q];
              T.a[q] += V.a[q];
              T.emin[q] = min(T.emin[q], V.emin[q]);
            }
            for (int d = 0; d < 3; ++d) {
              T.lo[d] = fminf(T.lo[d], V.lo[d]);
              T.hi[d] = fmaxf(T.hi[d], V.hi[d]);
            }
            T.ovf |= V.ovf;
          }
          lst[f - f0] = T;
        }
        team_sync(team, nw);
      }
    }
    __syncthreads();
    // ---- the level's decisions, a thread per node (the FP64 certification
    // runs on whole warps) ----
    for (int f = f0 + int(threadIdx.x); f < f1; f += kSubThreads) {
      DNode N = loc[f];
      const int c = N.count;
      if (c == 0) continue;  // an empty root (no particles) stays as it is
      SubWarpStats T = lst[f - f0];
      if (!decide_node(N, T.s, T.a, T.lo, T.hi, T.emin, T.ovf != 0, force_fallback, nd)) {
        // the reference's own sum: double, in array order (BGQCM.c:181-212)
        const int64_t o = N.offset;
        double x = 0, y = 0, z = 0, m = 0;
        for (int i = 0; i < c; ++i) {
          const float4 p = src[o + i];
          x = __dadd_rn(x, double(fmul_(p.w, p.x)));
          y = __dadd_rn(y, double(fmul_(p.w, p.y)));
          z = __dadd_rn(z, double(fmul_(p.w, p.z)));
          m = __dadd_rn(m, double(p.w));
        }
        N.xc[0] = __double2float_rn(__ddiv_rn(x, m));
        N.xc[1] = __double2float_rn(__ddiv_rn(y, m));
        N.xc[2] = __double2float_rn(__ddiv_rn(z, m));
        ++nfb;
      }
      loc[f] = N;
    }
    __syncthreads();
    // ---- partition at the centre of mass: a team per node ----
    for (int f = f0 + team; f < f1; f += nteams) {
      DNode N = loc[f];
      const int c = N.count;
      if (c == 0) continue;
      const int64_t o = N.offset;
      const int lo_off = int(o - roff);  // the node's first element in the subtree
      const int d = N.split_dim;
      if (d < 0) {
        // a leaf: its elements into the other buffer as well
        for (int e = tl; e < c; e += TN) {
          dst[o + e] = src[o + e];
          doid[o + e] = soid[o + e];
        }
        continue;
      }
      if (tl == 0) tflag[team] = 0;
      const float split = N.xc[d];
      const int share = (((c + nw - 1) / nw) + 31) & ~31;
      const int beg = wi * share, end = min(c, beg + share);
      int cl = 0;
      for (int e0 = beg; e0 < end; e0 += 32) {
        const int e = e0 + lane;
        const bool l = e < end && key_of(src[o + e], d) < split;
        cl += __popc(__ballot_sync(0xffffffffu, l));
      }
      if (lane == 0) wtot[warp] = cl;
      team_sync(team, nw);
      int rank = 0, nleft = 0;
      for (int w = 0; w < nw; ++w) {
        const int v = wtot[w0 + w];
        rank += w < wi ? v : 0;
        nleft += v;
      }
      for (int e0 = beg; e0 < end; e0 += 32) {
        const int e = e0 + lane;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        int32_t id = 0;
        if (e < end) {
          p = src[o + e];
          id = soid[o + e];
        }
        const bool l = e < end && key_of(p, d) < split;
        const unsigned bal = __ballot_sync(0xffffffffu, l);
        if (l) {
          const int q = rank + __popc(bal & below);
          dst[o + q] = p;
          doid[o + q] = id;
          sidx[lo_off + q] = e;
        } else if (e < end && e >= nleft) {
          // a right element at or after nleft: no swap touches it
          dst[o + e] = p;
          doid[o + e] = id;
        }
        rank += __popc(bal);
      }
      team_sync(team, nw);
      for (int e = tl; e < nleft; e += TN) {
        const float4 p = src[o + e];
        if (key_of(p, d) < split) continue;
        int q = e, steps = 0;
        bool bad = false;
        while (q < nleft && steps < kChainSteps) {
          const int nq = sidx[lo_off + q];
          if (nq <= q || nq >= c) {  // cannot happen for a valid partition
            bad = true;
            break;
          }
          q = nq;
          ++steps;
        }
        if (bad) {
          atomicExch(reinterpret_cast<int32_t *>(counters + C_ERR), 2);
          continue;
        }
        if (q < nleft) {
          tflag[team] = 1;
          continue;
        }
        dst[o + q] = p;
        doid[o + q] = soid[o + e];
      }
      team_sync(team, nw);
      if (tflag[team]) {
        // pointer jumping: afterwards sidx[q] is the end of the chain through q
        for (int round = 0;; ++round) {
          team_sync(team, nw);
          if (tl == 0) tflag[team] = 0;
          team_sync(team, nw);
          bool ch = false;
          for (int q = tl; q < nleft; q += TN) {
            const int j = sidx[lo_off + q];
            if (j != q && j < nleft) {  // j == q: a left element no swap moves
              sidx[lo_off + q] = sidx[lo_off + j];
              ch = true;
            }
          }
          if (__any_sync(0xffffffffu, ch) && lane == 0) tflag[team] = 1;
          team_sync(team, nw);
          if (!tflag[team]) break;
          if (round > 40) {  // cannot happen for a valid partition
            if (tl == 0) atomicExch(reinterpret_cast<int32_t *>(counters + C_ERR), 2);
            break;
          }
        }
        for (int e = tl; e < nleft; e += TN) {
          const float4 p = src[o + e];
          if (key_of(p, d) < split) continue;
          const int q = sidx[lo_off + e];
          if (q < nleft || q >= c) {
            atomicExch(reinterpret_cast<int32_t *>(counters + C_ERR), 2);
            continue;
          }
          dst[o + q] = p;
          doid[o + q] = soid[o + e];
        }
      }
      if (tl == 0) {
        N.nleft = nleft;
        loc[f] = N;
      }
      team_sync(team, nw);
    }
    __syncthreads();
    // ---- children: two per node split into two non-empty parts ----
    int base = f1;
    for (int c0 = f0; c0 < f1; c0 += kSubThreads) {
      const int f = c0 + int(threadIdx.x);
      int flag = 0;
      DNode N;
      if (f < f1) {
        N = loc[f];
        flag = (N.split_dim >= 0 && N.nleft > 0 && N.nleft < N.count) ? 1 : 0;
      }
      int tot = 0;
      const int rk = block_excl_scan(flag, sh_warp, &tot);
      if (f < f1) {
        if (flag) {
          const int cl = base + 2 * rk;
          N.cl = cl;
          N.cr = cl + 1;
          write_child(loc[cl], N, 0);
          write_child(loc[cl + 1], N, 1);
        } else {
          N.cl = N.cr = 0;
        }
        loc[f].cl = N.cl;
        loc[f].cr = N.cr;
      }
      base += 2 * tot;
    }
    if (threadIdx.x == 0) s_nsplit = (base - f1) / 2;
    __syncthreads();
    const int nsplit = s_nsplit;
    f0 = f1;
    f1 += 2 * nsplit;
    ++depth;
    if (threadIdx.x == 0) first[depth + 1] = f1;
    if (f1 > f0 && depth >= kSubDepth) {  // deeper than the bookkeeping holds
      if (threadIdx.x == 0) atomicExch(reinterpret_cast<int32_t *>(counters + C_ERR), 4);
      return;
    }
    {
      const float4 *t = src;
      src = dst;
      dst = const_cast<float4 *>(t);
      const int32_t *u = soid;
      soid = doid;
      doid = const_cast<int32_t *>(u);
    }
    __syncthreads();
  }
  if (nfb) atomicAdd((unsigned long long *)&counters[C_SUBFB], (unsigned long long)nfb);
  // per depth: first local node and count (depth 0 is the root)
  for (int dd = int(threadIdx.x); dd <= kSubDepth + 1; dd += kSubThreads)
    sub_first[int64_t(r) * (kSubDepth + 2) + dd] = dd <= depth + 1 ? first[min(dd, depth + 1)] : f1;
  for (int dd = 1 + int(threadIdx.x); dd <= kSubDepth; dd += kSubThreads)
    hist[int64_t(dd - 1) * nroots + r] = dd <= depth ? first[dd + 1] - first[dd] : 0;
}

// Node totals of every depth below the subtree roots, into tot[0..kSubDepth).
__global__ void k_subtree_totals(const int64_t *hist, int32_t nroots, int64_t *tot) {
  const int dd = blockIdx.x;
  int64_t v = 0;
  for (int32_t r = threadIdx.x; r < nroots; r += blockDim.x) v += hist[int64_t(dd) * nroots + r];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __shared__ int64_t part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t t = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += part[w];
    tot[dd] = t;
  }
}

// Copies every subtree node to its place among the levels: depth d below the
// roots is level nb-level + d, ordered by root (i.e. by offset) and, within a
// root, by the block's breadth-first order (also by offset).  pos holds the
// exclusive scan of hist (depth-major), ne the first index after the roots'
// level.
__global__ void k_subtree_place(DNode *nodes, int32_t nb, int32_t ne, const DNode *sub,
                                const int32_t *sub_first, const int64_t *pos) {
  __shared__ int fs[kSubDepth + 2];
  const int32_t r = int32_t(blockIdx.x);
  const int32_t nroots = ne - nb;
  for (int dd = threadIdx.x; dd <= kSubDepth + 1; dd += blockDim.x)
    fs[dd] = sub_first[int64_t(r) * (kSubDepth + 2) + dd];
  __syncthreads();
  const int32_t roff = nodes[nb + r].offset;
  const DNode *loc = sub + 2 * int64_t(roff);
  const int total = fs[kSubDepth + 1];
  auto depth_of = [&](int j) {
    int dd = 1;
    while (dd <= kSubDepth && fs[dd + 1] <= j) ++dd;
    return dd;
  };
  auto global = [&](int j, int dd) {
    return int32_t(ne + pos[int64_t(dd - 1) * nroots + r] + (j - fs[dd]));
  };
  for (int j = 1 + int(threadIdx.x); j < total; j += blockDim.x) {
    const int dd = depth_of(j);
    DNode N = loc[j];
    if (N.cl) {
      N.cl = global(N.cl, dd + 1);
      N.cr = global(N.cr, dd + 1);
    }
    nodes[global(j, dd)] = N;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DNode N = loc[0];
    if (N.cl) {
      N.cl = global(N.cl, 1);
      N.cr = global(N.cr, 1);
    }
    nodes[nb + r] = N;
  }
}

// 1 for nodes whose split produced two non-empty children.  (The element
// buffers alternate between levels; a leaf's elements are copied once into
// the next level's buffer by k_part_left, after which both buffers hold them
// and later levels write only inside splitting nodes.)
__global__ void k_split_flags(const DNode *nodes, int32_t nb, int32_t ne, int64_t *flag) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (nb + i >= ne) return;
  const DNode &N = nodes[nb + i];
  flag[i] = (N.split_dim >= 0 && N.nleft > 0 && N.nleft < N.count) ? 1 : 0;
}

__global__ void k_children(DNode *nodes, int32_t nb, int32_t ne, const int64_t *rank,
                           int64_t *maxcnt) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned m = 0;
  if (nb + i < ne) {
    const DNode &N = nodes[nb + i];
    if (N.split_dim >= 0 && N.nleft > 0 && N.nleft < N.count)
      m = unsigned(max(N.nleft, N.count - N.nleft));
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(reinterpret_cast<unsigned long long *>(maxcnt), m);
  if (nb + i >= ne) return;
  DNode &N = nodes[nb + i];
  if (!(N.split_dim >= 0 && N.nleft > 0 && N.nleft < N.count)) {
    N.cl = N.cr = 0;
    return;
  }
  const int32_t cl = ne + 2 * int32_t(rank[i]), cr = cl + 1;
  N.cl = cl;
  N.cr = cr;
  for (int s = 0; s < 2; ++s) {
    DNode &C = nodes[s == 0 ? cl : cr];
    C.count = s == 0 ? N.nleft : N.count - N.nleft;
    C.offset = s == 0 ? N.offset : N.offset + N.nleft;
    C.cl = C.cr = 0;
    for (int d = 0; d < 3; ++d) {
      C.xmin[d] = N.xmin[d];
      C.xmax[d] = N.xmax[d];
      C.xc[d] = 0.f;
    }
    C.tdr = 0.f;
    C.split_dim = -1;
    C.nleft = 0;
  }
}

// ---------------------------------------------------------------------------
// Pseudo-particles (RCBForceTree.cxx:519-569, 788-800, 856-889)
// ---------------------------------------------------------------------------
// The 12-point design (RCBForceTree.cxx:227-272): the icosahedron's vertices
// (0, +-b, +-a) and their cyclic permutations, a = 0.525731112119134,
// b = 0.85065080835204, in the reference's order.  Fixed: every tree reads
// it, whatever its point count (a monopole's one point sits at xc, offset 0).
#define HSR_IA 0.525731112119134f
#define HSR_IB 0.85065080835204f
__constant__ float c_design[12][3] = {
    {0, HSR_IB, HSR_IA},   {0, HSR_IB, -HSR_IA},  {HSR_IA, 0, HSR_IB},   {-HSR_IA, 0, HSR_IB},
    {HSR_IB, HSR_IA, 0},   {-HSR_IB, HSR_IA, 0},  {0, -HSR_IB, -HSR_IA}, {0, -HSR_IB, HSR_IA},
    {-HSR_IA, 0, -HSR_IB}, {HSR_IA, 0, -HSR_IB},  {-HSR_IB, -HSR_IA, 0}, {HSR_IB, -HSR_IA, 0}};
#undef HSR_IA
#undef HSR_IB

__device__ __forceinline__ float pptdr_(const DNode &t) {
  return smin_(fsub_(t.xmax[0], t.xc[0]),
               smin_(fsub_(t.xmax[1], t.xc[1]),
                     smin_(fsub_(t.xmax[2], t.xc[2]),
                           smin_(fsub_(t.xc[0], t.xmin[0]),
                                 smin_(fsub_(t.xc[1], t.xmin[1]), fsub_(t.xc[2], t.xmin[2]))))));
}

__device__ __forceinline__ void pppts_(int k, float tdr, const float *xc, float *px, float *py,
                                       float *pz) {
  for (int i = 0; i < k; ++i) {
    const float ex = k == 12 ? c_design[i][0] : 0.f, ey = k == 12 ? c_design[i][1] : 0.f,
                ez = k == 12 ? c_design[i][2] : 0.f;
    px[i] = fadd_(fmul_(tdr, ex), xc[0]);
    py[i] = fadd_(fmul_(tdr, ey), xc[1]);
    pz[i] = fadd_(fmul_(tdr, ez), xc[2]);
  }
}

// Adds `count` sources (x, y, z, m from src(i)) to the pseudo-particle masses.
template <typename Src>
__device__ void pp_accum_(int k, int32_t count, Src src, const float *xc, const float *px,
                          const float *py, const float *pz, float *ppm, float tdr) {
  const float K = float(k);
  const float odr0 = __fdiv_rn(1.0f, K);
  for (int32_t i = 0; i < count; ++i) {
    float sx, sy, sz, sm;
    src(i, sx, sy, sz, sm);
    const float xi = fsub_(sx, xc[0]), yi = fsub_(sy, xc[1]), zi = fsub_(sz, xc[2]);
    const float ri = __fsqrt_rn(norm2_(xi, yi, zi));
    for (int j = 0; j < k; ++j) {
      const float xj = fsub_(px[j], xc[0]), yj = fsub_(py[j], xc[1]), zj = fsub_(pz[j], xc[2]);
      const float rj2 = norm2_(xj, yj, zj);
      float odr1 = 0.f, odr2 = 0.f;
      if (rj2 != 0.f) {
        const float rj = __fsqrt_rn(rj2);
        const float aij = __fdiv_rn(fadd_(fadd_(fmul_(xi, xj), fmul_(yi, yj)), fmul_(zi, zj)),
                                    fmul_(ri, rj));
        const float rt = __fdiv_rn(ri, tdr);
        odr1 = fmul_(fmul_(__fdiv_rn(3.0f, K), rt), aij);
        const float a = fmul_(fmul_(__fdiv_rn(5.0f, K), rt), rt);
        const float b = fsub_(fmul_(fmul_(3.0f, aij), aij), 1.0f);
        odr2 = __double2float_rn(__dmul_rn(__dmul_rn(double(a), 0.5), double(b)));
      }
      ppm[j] = fadd_(ppm[j], fmul_(sm, fadd_(fadd_(odr0, odr1), odr2)));
    }
  }
}

// Node ranges of up to kTopLevels levels: level l is [b[l], b[l + 1]).
constexpr int kTopLevels = 48;
struct LevelSpan {
  int32_t b[kTopLevels + 1];
  int32_t n;
};

// Pseudo-particles of node t, its children done first.
__device__ void pseudo_node(DNode *nodes, int32_t t, const float4 *__restrict__ pos, float *ppm_all,
                            int k, float ppc, int32_t nd) {
  DNode &T = nodes[t];
  T.tdr = fmul_(ppc, pptdr_(T));
  float ppm[12];
  for (int j = 0; j < 12; ++j) ppm[j] = 0.f;
  float px[12], py[12], pz[12];
  if (T.cl == 0 && T.cr == 0) {
    // leaf by size: masses from its particles when it has more than k;
    // a leaf left by a failed split keeps zero masses (its children are empty)
    if (T.count <= nd && T.count > k) {
      const float4 *p = pos + T.offset;
      if (k == 1) {
        // the monopole's point is the centre of mass: every term's weight is
        // 1/1 + 0 + 0 (pp_accum_ with rj2 == 0), so the mass is the
        // sequential float sum of the particle masses
        float m = 0.f;
#pragma unroll 8
        for (int32_t i = 0; i < T.count; ++i) m = fadd_(m, fmul_(p[i].w, 1.0f));
        ppm[0] = m;
      } else {
        pppts_(k, T.tdr, T.xc, px, py, pz);
        pp_accum_(k, T.count, [&](int32_t i, float &x, float &y, float &z, float &m) {
          const float4 q = p[i];
          x = q.x; y = q.y; z = q.z; m = q.w;
        }, T.xc, px, py, pz, ppm, T.tdr);
      }
    }
  } else {
    pppts_(k, T.tdr, T.xc, px, py, pz);
    for (int s = 0; s < 2; ++s) {
      const DNode &C = nodes[s == 0 ? T.cl : T.cr];
      if (C.count <= 0) continue;
      if (C.count <= k) {
        const float4 *p = pos + C.offset;
        pp_accum_(k, C.count, [&](int32_t i, float &x, float &y, float &z, float &m) {
          const float4 q = p[i];
          x = q.x; y = q.y; z = q.z; m = q.w;
        }, T.xc, px, py, pz, ppm, T.tdr);
      } else {
        float cx[12], cy[12], cz[12];
        pppts_(k, C.tdr, C.xc, cx, cy, cz);
        const float *cm = ppm_all + int64_t(s == 0 ? T.cl : T.cr) * k;
        pp_accum_(k, k, [&](int32_t i, float &x, float &y, float &z, float &m) {
          x = cx[i]; y = cy[i]; z = cz[i]; m = cm[i];
        }, T.xc, px, py, pz, ppm, T.tdr);
      }
    }
  }
  for (int j = 0; j < k; ++j) ppm_all[int64_t(t) * k + j] = ppm[j];
}

// Pseudo-particles of the nodes [lb, le), a warp per node.  A monopole leaf's
// mass is the sequential float sum of its particles' masses: the warp loads
// 32 at a time (coalesced) and every lane adds them in order from shuffles.
// Other nodes: lane 0.
__global__ void k_pseudo(DNode *nodes, int32_t lb, int32_t le, const float4 *__restrict__ pos,
                         float *ppm_all, int k, float ppc, int32_t nd) {
  const int32_t t = lb + int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= le) return;  // whole warps
  DNode &T = nodes[t];
  if (k == 1 && T.cl == 0 && T.cr == 0 && T.count <= nd && T.count > 1) {
    const float *w = reinterpret_cast<const float *>(pos + T.offset) + 3;
    const int32_t c = T.count;
    float m = 0.f;
    for (int32_t i0 = 0; i0 < c; i0 += 32) {
      const float v = i0 + lane < c ? w[4 * (i0 + lane)] : 0.f;
      const int nv = min(32, c - i0);
      for (int j = 0; j < nv; ++j) m = fadd_(m, fmul_(__shfl_sync(0xffffffffu, v, j), 1.0f));
    }
    if (lane == 0) {
      T.tdr = fmul_(ppc, pptdr_(T));
      ppm_all[t] = m;
    }
    return;
  }
  if (lane == 0) pseudo_node(nodes, t, pos, ppm_all, k, ppc, nd);
}

// The top levels' pseudo-particles in one block, deepest level first, a
// thread per node (every level here has at most blockDim.x nodes).
__global__ void __launch_bounds__(1024)
    k_pseudo_top(DNode *nodes, LevelSpan lv, const float4 *__restrict__ pos, float *ppm_all, int k,
                 float ppc, int32_t nd) {
  for (int l = lv.n - 1; l >= 0; --l) {
    for (int32_t t = lv.b[l] + int32_t(threadIdx.x); t < lv.b[l + 1]; t += int32_t(blockDim.x))
      pseudo_node(nodes, t, pos, ppm_all, k, ppc, nd);
    __syncthreads();  // the next level up reads these nodes
  }
}

// Position table: particles, then every node's pseudo-particles.
__global__ void k_table_pseudo(const DNode *nodes, int32_t nnodes, const float *ppm_all, int k,
                               float4 *table, int64_t n) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnodes) return;
  const DNode &T = nodes[t];
  float px[12], py[12], pz[12];
  pppts_(k, T.tdr, T.xc, px, py, pz);
  for (int j = 0; j < k; ++j)
    table[n + int64_t(t) * k + j] = make_float4(px[j], py[j], pz[j], ppm_all[int64_t(t) * k + j]);
}

// ---------------------------------------------------------------------------
// Processed leaves (calcInternodeForces, RCBForceTree.cxx:1150-1197): leaves
// inside the force box, in the reference's DFS order, which visits the right
// child first, i.e. by decreasing particle offset.
// ---------------------------------------------------------------------------
__global__ void k_mark_leaves(const DNode *nodes, int32_t nnodes, TreeConfig cfg, int64_t n,
                              int64_t *leaf_at) {
  const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnodes) return;
  const DNode &T = nodes[t];
  if (T.cl != 0 || T.cr != 0 || T.count <= 0) return;
  bool inside = true;
  for (int i = 0; i < 3; ++i)
    inside &= (T.xmax[i] < cfg.max_force[i] && T.xmax[i] > cfg.min_force[i]) ||
              (T.xmin[i] < cfg.max_force[i] && T.xmin[i] > cfg.min_force[i]);
  if (inside) leaf_at[n - 1 - T.offset] = t;  // reversed: decreasing offset
}

__global__ void k_leaf_flags(const int64_t *leaf_at, int64_t n, int64_t *flag) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = leaf_at[i] >= 0;
}

__global__ void k_leaf_compact(const int64_t *leaf_at, const int64_t *pos_of, int64_t n,
                               int32_t *leaf_ids) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && leaf_at[i] >= 0) leaf_ids[pos_of[i]] = int32_t(leaf_at[i]);
}

// ---------------------------------------------------------------------------
// Interaction lists (calcInternodeForce, RCBForceTree.cxx:923-1144), one
// thread per processed leaf; a counting pass and a writing pass.
// ---------------------------------------------------------------------------
// MODE 0: counts (segments and entries per leaf); 1: writes the segments at
// seg_base / list_base; 2: counts and writes the first kLocalSegs segments
// of each leaf into its own region (dst relative to the leaf's list),
// flagging leaves with more in counters[C_SEGOVF].
template <int MODE>
__global__ void k_walk(const DNode *__restrict__ nodes, int32_t nnodes, const int32_t *leaf_ids,
                       int64_t nleaves, TreeConfig cfg, int64_t n, int64_t *seg_cnt, int64_t *list_len,
                       const int64_t *seg_base, const int64_t *list_base, SegDesc *segs,
                       int32_t *err, int64_t *counters) {
  constexpr bool WRITE = MODE == 1;
  const int64_t li = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (li >= nleaves) return;
  const int32_t tl = leaf_ids[li];
  const DNode T = nodes[tl];
  const float fsr = cfg.fsrrmax;
  const float fsr2 = fmul_(fsr, fsr);
  const float tan_oa = cfg.tan_oa;
  const int k = cfg.tdpts;
  int32_t stack[kWalkStack];
  int sp = 0;
  int64_t nseg = 0, len = 0;
  const int64_t sb = WRITE ? seg_base[li] : 0, lb = WRITE ? list_base[li] : 0;
  auto emit = [&](int64_t start, int64_t count) {
    if (count <= 0) return;
    if (WRITE) segs[sb + nseg] = SegDesc{int32_t(start), int32_t(count), lb + len};
    if (MODE == 2 && nseg < kLocalSegs)
      segs[li * kLocalSegs + nseg] = SegDesc{int32_t(start), int32_t(count), len};
    ++nseg;
    len += count;
  };
  auto push = [&](int32_t v) {
    if (sp < kWalkStack) stack[sp++] = v;
    else atomicExch(err, 1);
  };
  auto close_to = [&](const DNode &C) {
    for (int i = 0; i < 3; ++i) {
      float dist = 0.f;
      if (T.xmax[i] < C.xmin[i]) dist = fsub_(C.xmin[i], T.xmax[i]);
      else if (T.xmin[i] > C.xmax[i]) dist = fsub_(T.xmin[i], C.xmax[i]);
      if (dist > fsr) return false;
    }
    return true;
  };
  push(0);
  int64_t pops = 0;
  while (sp > 0) {
    if (++pops > int64_t(nnodes) + 1) {  // a tree walk visits each node at most once
      atomicExch(err, 3);
      break;
    }
    const int32_t t = stack[--sp];
    if (t < 0 || t >= nnodes) {
      atomicExch(err, 3);
      break;
    }
    const DNode Q = nodes[t];
    if (Q.cl >= nnodes || Q.cr >= nnodes) {
      atomicExch(err, 3);
      break;
    }
    if (t != tl && Q.offset <= T.offset && T.offset + T.count <= Q.offset + Q.count) {
      if (Q.cl != tl && Q.cl > 0 && nodes[Q.cl].count > 0) push(Q.cl);
      if (Q.cr != tl && Q.cr > 0 && nodes[Q.cr].count > 0) push(Q.cr);
      continue;
    }
    const float dx = fsub_(Q.xc[0], T.xc[0]), dy = fsub_(Q.xc[1], T.xc[1]),
                dz = fsub_(Q.xc[2], T.xc[2]);
    const float dist2 = norm2_(dx, dy, dz);
    const float sx = fsub_(Q.xmax[0], Q.xmin[0]), sy = fsub_(Q.xmax[1], Q.xmin[1]),
                sz = fsub_(Q.xmax[2], Q.xmin[2]);
    const float l2 = smin_(fmul_(sx, sx), smin_(fmul_(sy, sy), fmul_(sz, sz)));
    const float dtt2 = fmul_(fmul_(dist2, tan_oa), tan_oa);
    bool big = l2 > dtt2;
    for (int i = 0; i < 2 && !big; ++i)
      for (int j = 0; j < 2 && !big; ++j) {
        const float x1 = fsub_((i == 0 ? Q.xmin : Q.xmax)[0], T.xc[0]);
        const float y1 = fsub_((j == 0 ? Q.xmin : Q.xmax)[1], T.xc[1]);
        const float z1 = fsub_(Q.xmin[2], T.xc[2]);
        const float x2 = fsub_((i == 0 ? Q.xmax : Q.xmin)[0], T.xc[0]);
        const float y2 = fsub_((j == 0 ? Q.xmax : Q.xmin)[1], T.xc[1]);
        const float z2 = fsub_(Q.xmax[2], T.xc[2]);
        big = norm2_(fsub_(x1, x2), fsub_(y1, y2), fsub_(z1, z2)) > dtt2;
      }
    if (!big) {
      if (dist2 > fsr2) continue;
      if (Q.count <= k) emit(Q.offset, Q.count);
      else emit(n + int64_t(t) * k, k);
      continue;
    }
    if (Q.cr == 0 && Q.cl == 0) {
      emit(Q.offset, Q.count);
      continue;
    }
    if (Q.cl > 0 && nodes[Q.cl].count > 0 && close_to(nodes[Q.cl])) push(Q.cl);
    if (Q.cr > 0 && nodes[Q.cr].count > 0 && close_to(nodes[Q.cr])) push(Q.cr);
  }
  emit(T.offset, T.count);
  if (!WRITE) {
    seg_cnt[li] = nseg;
    list_len[li] = len;
  }
  if (MODE == 2 && nseg > kLocalSegs) atomicExch((unsigned long long *)&counters[C_SEGOVF], 1ull);
}

// The one-pass walk's per-leaf regions packed leaf after leaf, with each
// segment's destination made absolute.
__global__ void k_pack_segs(const SegDesc *__restrict__ local, const int64_t *seg_cnt,
                            const int64_t *seg_base, const int64_t *list_base, int64_t nleaves,
                            SegDesc *__restrict__ segs) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t li = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; li < nleaves;
       li += warps) {
    const int64_t c = seg_cnt[li], sb = seg_base[li], lb = list_base[li];
    for (int64_t q = lane; q < c; q += 32) {
      SegDesc d = local[li * kLocalSegs + q];
      d.dst += lb;
      segs[sb + q] = d;
    }
  }
}

// Expands each leaf's segments into the index array at the leaf's list_base,
// keeping only the entries within sqrt(cull2) of the leaf's box: the others
// are farther than the cutoff from every particle of the leaf, so the
// reference's mask gives them exactly 0.  Warp per leaf: the leaf's box as
// centre and half-width (widened by 4 ulps of
// the coordinates, as in the batched kernel), then its segments 32 entries at
// a time, compacting the kept entries by ballot.
__global__ void k_expand_pruned(const SegDesc *__restrict__ segs,
                                const int64_t *__restrict__ seg_base,
                                const int64_t *__restrict__ seg_cnt,
                                const int64_t *__restrict__ list_base,
                                const DNode *__restrict__ nodes,
                                const int32_t *__restrict__ leaf_ids, int64_t nleaves,
                                const float4 *__restrict__ table, float cull2,
                                int32_t *__restrict__ idx, int64_t *__restrict__ kept) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int64_t warps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t li = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; li < nleaves;
       li += warps) {
    const DNode &T = nodes[leaf_ids[li]];
    const float lox = T.xmin[0], loy = T.xmin[1], loz = T.xmin[2];
    const float hix = T.xmax[0], hiy = T.xmax[1], hiz = T.xmax[2];
    const float hx = fmaf(fmaxf(fabsf(lox), fabsf(hix)), 4.8e-7f, 0.5f * (hix - lox));
    const float hy = fmaf(fmaxf(fabsf(loy), fabsf(hiy)), 4.8e-7f, 0.5f * (hiy - loy));
    const float hz = fmaf(fmaxf(fabsf(loz), fabsf(hiz)), 4.8e-7f, 0.5f * (hiz - loz));
    const float cx = 0.5f * (lox + hix), cy = 0.5f * (loy + hiy), cz = 0.5f * (loz + hiz);
    int32_t *out = idx + list_base[li];
    int64_t nk = 0;
    const int64_t s0 = seg_base[li], s1 = s0 + seg_cnt[li];
    for (int64_t q = s0; q < s1; ++q) {
      const SegDesc S = segs[q];
      for (int k0 = 0; k0 < S.count; k0 += 32) {
        const int k = k0 + lane;
        bool keep = false;
        if (k < S.count) {
          const float4 J = table[S.start + k];
          const float dx = fmaxf(fabsf(J.x - cx) - hx, 0.f);
          const float dy = fmaxf(fabsf(J.y - cy) - hy, 0.f);
          const float dz = fmaxf(fabsf(J.z - cz) - hz, 0.f);
          keep = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < cull2;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) out[nk + __popc(m & below)] = S.start + k;
        nk += __popc(m);
      }
    }
    if (lane == 0) kept[li] = nk;
  }
}


__global__ void k_leaf_desc(const DNode *nodes, const int32_t *leaf_ids, int64_t nleaves,
                            const int64_t *list_len, const int64_t *kept_len,
                            const int64_t *list_base, LeafDesc *ld, int64_t *counters) {
  const int64_t li = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  long long pairs = 0, padded = 0, mx = 0;
  if (li < nleaves) {
    const DNode &T = nodes[leaf_ids[li]];
    LeafDesc d{};
    d.offset = T.offset;
    d.count = T.count;
    d.list_len = int32_t(list_len[li]);
    d.kept_len = int32_t(kept_len ? kept_len[li] : list_len[li]);
    d.list_begin = list_base[li];
    ld[li] = d;
    pairs = (long long)T.count * list_len[li];
    padded = (long long)((T.count + 31) / 32) * 32 * d.kept_len;
    mx = d.kept_len;
  }
  for (int o = 16; o > 0; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    padded += __shfl_xor_sync(0xffffffffu, padded, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd((unsigned long long *)&counters[C_PAIRS], (unsigned long long)pairs);
    atomicAdd((unsigned long long *)&counters[C_PADDED], (unsigned long long)padded);
    atomicMax((long long *)&counters[C_MAXLEN], mx);
  }
}

// ---------------------------------------------------------------------------
// Groups of <= 32 spatially close particles per processed leaf (Morton order
// inside the leaf's box) and the batched kernel's work items.
// ---------------------------------------------------------------------------
constexpr int kGroupSort = 1024;
constexpr int kGW = 256;     // leaves up to this size are grouped by one warp
constexpr int kGWarps = 4;   // warps (leaves) per block of k_groups_warp
constexpr int kGroupThreads = 256;

// Order-preserving map of a float to an unsigned integer.
__device__ __forceinline__ uint32_t f2o(float v) {
  const uint32_t b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Splits each processed leaf into groups of G particles (the last one
// shorter) by recursive median splits along the longest axis, left parts a
// multiple of G: the particles of a group are close, so the batched kernel's box test
// keeps few list entries.  Every level sorts all segments of the leaf at once
// by (segment, coordinate along the segment's longest axis).
__global__ void __launch_bounds__(kGroupThreads)
    k_groups(const DNode *nodes, const int32_t *leaf_ids, int64_t nleaves,
             const float4 *__restrict__ pos, int32_t *gidx, int G) {
  __shared__ uint64_t key[kGroupSort];
  __shared__ int32_t val[kGroupSort];
  __shared__ int32_t seg_a[kGroupSort / 16 + 1], seg_c[kGroupSort / 16 + 1];
  __shared__ uint32_t seg_lo[3][kGroupSort / 16 + 1], seg_hi[3][kGroupSort / 16 + 1];
  __shared__ int nseg_s, more_s;
  const int64_t li = blockIdx.x;
  if (li >= nleaves) return;
  const DNode &T = nodes[leaf_ids[li]];
  const int32_t c = T.count;
  if (c <= kGW) return;  // k_groups_warp
  if (c > kGroupSort) {
    for (int32_t i = threadIdx.x; i < c; i += blockDim.x) gidx[T.offset + i] = T.offset + i;
    return;
  }
  int m = 1;
  while (m < c) m <<= 1;
  // padding slots sort last but pass through the upper half on the way
  for (int i = threadIdx.x; i < m; i += blockDim.x) val[i] = i < c ? T.offset + i : -1;
  if (threadIdx.x == 0) {
    seg_a[0] = 0;
    seg_c[0] = c;
    nseg_s = 1;
  }
  __syncthreads();
  for (int level = 0; level < 16; ++level) {
    const int nseg = nseg_s;
    // boxes of the segments that still need a split
    for (int q = threadIdx.x; q < nseg; q += blockDim.x)
      for (int d = 0; d < 3; ++d) {
        seg_lo[d][q] = 0xffffffffu;
        seg_hi[d][q] = 0u;
      }
    __syncthreads();
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      int q = 0;
      while (q + 1 < nseg && seg_a[q + 1] <= i) ++q;
      if (seg_c[q] <= G) continue;
      const float4 p = pos[val[i]];
      const uint32_t o[3] = {f2o(p.x), f2o(p.y), f2o(p.z)};
      for (int d = 0; d < 3; ++d) {
        atomicMin(&seg_lo[d][q], o[d]);
        atomicMax(&seg_hi[d][q], o[d]);
      }
    }
    __syncthreads();
    // sort key: segment, then the coordinate on the segment's longest axis
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      uint64_t kv = ~0ull;
      if (i < c) {
        int q = 0;
        while (q + 1 < nseg && seg_a[q + 1] <= i) ++q;
        uint32_t ko = 0;
        if (seg_c[q] > G) {
          float ext[3];
          for (int d = 0; d < 3; ++d) ext[d] = o2f(seg_hi[d][q]) - o2f(seg_lo[d][q]);
          const int ax = (ext[0] >= ext[1] && ext[0] >= ext[2]) ? 0 : (ext[1] >= ext[2] ? 1 : 2);
          const float4 p = pos[val[i]];
          ko = f2o(ax == 0 ? p.x : (ax == 1 ? p.y : p.z));
        } else {
          ko = uint32_t(i);  // settled segments keep their order
        }
        kv = (uint64_t(q) << 32) | ko;
      }
      key[i] = kv;
    }
    __syncthreads();
    for (int size = 2; size <= m; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
          const int j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const uint64_t ka = key[i], kb = key[j];
            if ((ka > kb) == up) {
              key[i] = kb;
              key[j] = ka;
              const int32_t t = val[i];
              val[i] = val[j];
              val[j] = t;
            }
          }
        }
        __syncthreads();
      }
    // split every segment above G at G * ceil(groups / 2)
    if (threadIdx.x == 0) {
      int n2 = 0;
      int32_t na[kGroupSort / 16 + 1], nc[kGroupSort / 16 + 1];
      int more = 0;
      for (int q = 0; q < nseg; ++q) {
        const int32_t a0 = seg_a[q], c0 = seg_c[q];
        if (c0 <= G) {
          na[n2] = a0;
          nc[n2++] = c0;
          continue;
        }
        const int32_t ng = (c0 + G - 1) / G, left = G * ((ng + 1) / 2);
        na[n2] = a0;
        nc[n2++] = left;
        na[n2] = a0 + left;
        nc[n2++] = c0 - left;
        more |= left > G || c0 - left > G;
      }
      for (int q = 0; q < n2; ++q) {
        seg_a[q] = na[q];
        seg_c[q] = nc[q];
      }
      nseg_s = n2;
      more_s = more;
    }
    __syncthreads();
    if (!more_s) break;
  }
  for (int i = threadIdx.x; i < c; i += blockDim.x) gidx[T.offset + i] = val[i];
}

// Warp-per-leaf grouping for leaves of at most kGW particles (the usual
// case; larger leaves take k_groups).  Same median splits as k_groups: per
// level, every segment above G particles is sorted along its longest axis by
// ranking (each element counts the keys below its own, ties by position) and
// split at G * ceil(groups / 2).
__global__ void __launch_bounds__(32 * kGWarps)
    k_groups_warp(const DNode *nodes, const int32_t *leaf_ids, int64_t nleaves,
                  const float4 *__restrict__ pos, int32_t *gidx, int G) {
  __shared__ float key[kGWarps][kGW];
  __shared__ int32_t val[kGWarps][2][kGW];
  __shared__ uint8_t segid[kGWarps][kGW];
  __shared__ int16_t seg_a[kGWarps][kGW / 16 + 1], seg_c[kGWarps][kGW / 16 + 1];
  __shared__ int8_t seg_ax[kGWarps][kGW / 16 + 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t li = int64_t(blockIdx.x) * kGWarps + w;
  if (li >= nleaves) return;
  const DNode &T = nodes[leaf_ids[li]];
  const int c = T.count;
  if (c <= 0 || c > kGW) return;
  if (c <= G) {
    for (int i = lane; i < c; i += 32) gidx[T.offset + i] = T.offset + i;
    return;
  }
  for (int i = lane; i < c; i += 32) {
    val[w][0][i] = T.offset + i;
    segid[w][i] = 0;
  }
  int nseg = 1;
  if (lane == 0) {
    seg_a[w][0] = 0;
    seg_c[w][0] = int16_t(c);
  }
  __syncwarp();
  int cur = 0;
  for (int level = 0; level < 16; ++level) {
    // longest axis of every segment above G
    bool any = false;
    for (int q = 0; q < nseg; ++q) {
      const int a0 = seg_a[w][q], c0 = seg_c[w][q];
      if (c0 <= G) continue;
      any = true;
      float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (int i = a0 + lane; i < a0 + c0; i += 32) {
        const float4 p = pos[val[w][cur][i]];
        lo[0] = fminf(lo[0], p.x); hi[0] = fmaxf(hi[0], p.x);
        lo[1] = fminf(lo[1], p.y); hi[1] = fmaxf(hi[1], p.y);
        lo[2] = fminf(lo[2], p.z); hi[2] = fmaxf(hi[2], p.z);
      }
      for (int d = 0; d < 3; ++d) {
        lo[d] = warp_min(lo[d]);
        hi[d] = warp_max(hi[d]);
      }
      const float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
      if (lane == 0) seg_ax[w][q] = int8_t((e0 >= e1 && e0 >= e2) ? 0 : (e1 >= e2 ? 1 : 2));
    }
    if (!any) break;
    __syncwarp();
    for (int i = lane; i < c; i += 32) {
      const int q = segid[w][i];
      float k = 0.f;
      if (seg_c[w][q] > G) {
        const float4 p = pos[val[w][cur][i]];
        const int ax = seg_ax[w][q];
        k = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
      }
      key[w][i] = k;
    }
    __syncwarp();
    for (int i = lane; i < c; i += 32) {
      const int q = segid[w][i];
      const int a0 = seg_a[w][q], c0 = seg_c[w][q];
      int np = i;
      if (c0 > G) {
        const float ki = key[w][i];
        int r = 0;
        for (int j = a0; j < a0 + c0; ++j) {
          const float kj = key[w][j];
          r += (kj < ki) || (kj == ki && j < i);
        }
        np = a0 + r;
      }
      val[w][cur ^ 1][np] = val[w][cur][i];
    }
    __syncwarp();
    cur ^= 1;
    // split every segment above G at G * ceil(groups / 2)
    if (lane == 0) {
      int16_t na[kGW / 16 + 1], nc[kGW / 16 + 1];
      int n2 = 0;
      for (int q = 0; q < nseg; ++q) {
        const int a0 = seg_a[w][q], c0 = seg_c[w][q];
        if (c0 <= G) {
          na[n2] = int16_t(a0);
          nc[n2++] = int16_t(c0);
          continue;
        }
        const int ng = (c0 + G - 1) / G, left = G * ((ng + 1) / 2);
        na[n2] = int16_t(a0);
        nc[n2++] = int16_t(left);
        na[n2] = int16_t(a0 + left);
        nc[n2++] = int16_t(c0 - left);
      }
      for (int q = 0; q < n2; ++q) {
        seg_a[w][q] = na[q];
        seg_c[w][q] = nc[q];
      }
      seg_ax[w][kGW / 16] = int8_t(n2);  // count, read back below
    }
    __syncwarp();
    nseg = seg_ax[w][kGW / 16];
    for (int q = 0; q < nseg; ++q)
      for (int i = seg_a[w][q] + lane; i < seg_a[w][q] + seg_c[w][q]; i += 32) segid[w][i] = uint8_t(q);
    __syncwarp();
  }
  for (int i = lane; i < c; i += 32) gidx[T.offset + i] = val[w][cur][i];
}

__device__ __forceinline__ int len_bucket(int64_t len) {
  // 32 buckets, longest lists first
  const int b = 63 - __clzll((unsigned long long)max64(len, 1));
  return 31 - min(31, b);
}

__global__ void k_item_hist(const LeafDesc *ld, int64_t nleaves, int64_t jsplit, int G,
                            int64_t *counters) {
  const int64_t li = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (li >= nleaves) return;
  const LeafDesc &L = ld[li];
  const int64_t nch = max64(1, (L.kept_len + jsplit - 1) / jsplit);
  const int64_t items = int64_t((L.count + G - 1) / G) * nch;
  atomicAdd((unsigned long long *)&counters[C_BUCKET + len_bucket(min64(L.kept_len, jsplit))],
            (unsigned long long)items);
}

__global__ void k_item_bases(int64_t *counters) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t run = 0;
  for (int b = 0; b < 32; ++b) {
    counters[C_FILL + b] = run;
    run += counters[C_BUCKET + b];
  }
  counters[C_NITEMS] = run;
}

__global__ void k_item_fill(const LeafDesc *ld, int64_t nleaves, int64_t jsplit, int G,
                            int64_t *counters, PairItem *items) {
  const int64_t li = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (li >= nleaves) return;
  const LeafDesc &L = ld[li];
  const int64_t nch = max64(1, (L.kept_len + jsplit - 1) / jsplit);
  const int32_t ng = (L.count + G - 1) / G;
  const int64_t items_n = int64_t(ng) * nch;
  if (items_n == 0) return;
  const int b = len_bucket(min64(L.kept_len, jsplit));
  int64_t at = int64_t(atomicAdd((unsigned long long *)&counters[C_FILL + b],
                                 (unsigned long long)items_n));
  for (int32_t g = 0; g < ng; ++g)
    for (int64_t c = 0; c < nch; ++c) {
      PairItem it{};
      it.j_begin = L.list_begin + c * jsplit;
      it.j_len = int32_t(min64(jsplit, L.kept_len - c * jsplit));
      it.g_begin = L.offset + G * g;
      it.g_count = min(G, L.count - G * g);
      it.flags = nch > 1 ? 1 : 0;
      items[at++] = it;
    }
}

// ---------------------------------------------------------------------------
// Gathers and packing
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_gather(const T *__restrict__ in, const int32_t *__restrict__ perm, T *out,
                         int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = in[perm[i]];
}

// The three velocity components into tree order, perm read once:
// out[d n + i] = in_d[perm[i]].
__global__ void k_gather3_f32(const float *__restrict__ a, const float *__restrict__ b,
                              const float *__restrict__ c, const int32_t *__restrict__ perm,
                              float *out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int32_t j = perm[i];
    out[i] = a[j];
    out[n + i] = b[j];
    out[2 * n + i] = c[j];
  }
}

// Every permuted output but the velocities in one pass: positions and masses
// from the tree-ordered table, phi, id and mask through perm.
__global__ void k_outputs(const float4 *__restrict__ table, const float *__restrict__ phi,
                          const int64_t *__restrict__ id, const uint16_t *__restrict__ mask,
                          const int32_t *__restrict__ perm, float *x, float *y, float *z, float *m,
                          float *ophi, int64_t *oid, uint16_t *omask, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int32_t j = perm[i];
    const float4 p = table[i];
    const float f = phi[j];
    const int64_t d = id[j];
    const uint16_t k = mask[j];
    x[i] = p.x;
    y[i] = p.y;
    z[i] = p.z;
    m[i] = p.w;
    ophi[i] = f;
    oid[i] = d;
    omask[i] = k;
  }
}

__global__ void k_pack4(const float *x, const float *y, const float *z, const float *m, float4 *out,
                        int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = make_float4(x[i], y[i], z[i], m[i]);
}

__global__ void k_scatter_f32(const float *__restrict__ in, const int32_t *__restrict__ perm,
                              float *out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[perm[i]] = in[i];
}

__global__ void k_scatter_add_f32(const float *__restrict__ in, const int32_t *__restrict__ perm,
                                  float *out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    out[perm[i]] += in[i];
}

// acc holds, per node, sum over it and its ancestors of xbar_P / M_P.
// Monopole pseudo-particle gradients passed to the particles: a warp per
// leaf sums xbar / m of the nodes on its root-to-leaf path (root first, the
// same float additions as a level-by-level top-down pass) and adds m_k times
// the sum to each of its particles.  The path follows the child holding the
// leaf's offset (left when below offset + nleft).
__global__ void k_adj_paths(const DNode *__restrict__ nodes, int32_t nnodes,
                            const float4 *__restrict__ table, int64_t n, float *xbx, float *xby,
                            float *xbz, int32_t *err) {
  const int32_t leaf = int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (leaf >= nnodes) return;  // whole warps
  const DNode &L = nodes[leaf];
  if (L.cl != 0 || L.cr != 0 || L.count <= 0) return;
  const int32_t lo = L.offset;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  int32_t t = 0;
  for (int depth = 0;; ++depth) {
    const float m = table[n + t].w;
    const float inv = m != 0.f ? 1.f / m : 0.f;
    a0 = a0 + xbx[n + t] * inv;
    a1 = a1 + xby[n + t] * inv;
    a2 = a2 + xbz[n + t] * inv;
    if (t == leaf) break;
    const DNode &T = nodes[t];
    const int32_t c = lo < T.offset + T.nleft ? T.cl : T.cr;
    if (c <= 0 || c >= nnodes || depth > 256) {  // cannot happen in a valid tree
      if (lane == 0) atomicExch(err, 5);
      return;
    }
    t = c;
  }
  if (a0 == 0.f && a1 == 0.f && a2 == 0.f) return;
  for (int32_t i = lane; i < L.count; i += 32) {
    const int32_t k = L.offset + i;
    const float m = table[k].w;
    xbx[k] += m * a0;
    xby[k] += m * a1;
    xbz[k] += m * a2;
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the 12-point pseudo-particles (RCBForceTree.cxx:519-568,
// :786-799, :855-889).  A node's point a sits at p_a = xc + tdr e_a and has
// the mass ppm_a = sum_s m_s f_a(y_s - xc, tdr) over its sources s (its
// particles, or each child's particles or points), in exact arithmetic
//   f_a(d, tdr) = 1/K + (3/K) (d.e_a)/tdr + (5/(2K)) (3 (d.e_a)^2 - |d|^2)/tdr^2
// (1/K alone for tdr = 0); tdr = ppc x (the least distance from xc to a face
// of the node's box) and xc the node's centre of mass.  Given the cotangents
// of every point's position (xbar) and mass (mbar), the nodes are taken top
// down: each passes its points' cotangents to its sources (a child's points
// before that child is taken), to its xc and to its tdr; the tdr cotangent
// then goes to the particle on the face pptdr took, and every xc cotangent to
// the node's particles (m_i / M).
// ---------------------------------------------------------------------------
constexpr int kQuad = 12;

// A warp per node of level [lb, le).
__global__ void k_quad_adj_level(const DNode *__restrict__ nodes, int32_t lb, int32_t le,
                                 const float4 *__restrict__ table, int64_t n, int32_t nd,
                                 float *xbx, float *xby, float *xbz, float *mb, float *xcbar,
                                 float *tdrbar) {
  __shared__ float sx[8][kQuad][4];  // per warp: the node's points' cotangents (x, y, z, m)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int32_t t = lb + int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  if (t >= le) return;  // whole warps
  const DNode &T = nodes[t];
  const int32_t c = T.count;
  const bool leaf = T.cl == 0 && T.cr == 0;
  // no points used (a node of at most 12 particles is listed by its
  // particles), or a leaf left by a failed split (massless points, no sources)
  if (c <= kQuad || (leaf && c > nd)) return;
  const int64_t pb = n + int64_t(kQuad) * t;
  if (lane < kQuad) {
    sx[w][lane][0] = xbx[pb + lane];
    sx[w][lane][1] = xby[pb + lane];
    sx[w][lane][2] = xbz[pb + lane];
    sx[w][lane][3] = mb[pb + lane];
  }
  __syncwarp();
  const float xc0 = T.xc[0], xc1 = T.xc[1], xc2 = T.xc[2], tdr = T.tdr;
  const float K = float(kQuad);
  float gx = 0.f, gy = 0.f, gz = 0.f, gt = 0.f;  // xc and tdr cotangents
  // p_a = xc + tdr e_a
  if (lane < kQuad) {
    const float ax = sx[w][lane][0], ay = sx[w][lane][1], az = sx[w][lane][2];
    gx += ax;
    gy += ay;
    gz += az;
    gt += ax * c_design[lane][0] + ay * c_design[lane][1] + az * c_design[lane][2];
  }
  // one source at table index j: its cotangents, and its share of xc's and tdr's
  auto source = [&](int64_t j, bool point) {
    const float4 y = table[j];
    const float dx = y.x - xc0, dy = y.y - xc1, dz = y.z - xc2;
    float fx = 0.f, fy = 0.f, fz = 0.f, ft = 0.f, fm = 0.f;
    if (tdr == 0.f) {
      for (int a = 0; a < kQuad; ++a) fm += sx[w][a][3];
      fm *= 1.f / K;
    } else {
      const float it = 1.f / tdr, it2 = it * it;
      const float d2 = dx * dx + dy * dy + dz * dz;
      for (int a = 0; a < kQuad; ++a) {
        const float ex = c_design[a][0], ey = c_design[a][1], ez = c_design[a][2];
        const float M = sx[w][a][3];
        const float q = dx * ex + dy * ey + dz * ez;
        const float p2 = 3.f * q * q - d2;
        fm += M * (1.f / K + (3.f / K) * q * it + (2.5f / K) * p2 * it2);
        // d f / d d = (3/K) e / tdr + (5/(2K)) (6 q e - 2 d) / tdr^2
        const float ce = M * ((3.f / K) * it + (15.f / K) * q * it2);
        const float cd = -M * (5.f / K) * it2;
        fx += ce * ex + cd * dx;
        fy += ce * ey + cd * dy;
        fz += ce * ez + cd * dz;
        // d f / d tdr = -(3/K) q / tdr^2 - (5/K) (3 q^2 - |d|^2) / tdr^3
        ft -= M * ((3.f / K) * q * it2 + (5.f / K) * p2 * it2 * it);
      }
    }
    const float m = y.w;
    xbx[j] += m * fx;
    xby[j] += m * fy;
    xbz[j] += m * fz;
    gx -= m * fx;
    gy -= m * fy;
    gz -= m * fz;
    gt += m * ft;
    if (point) mb[j] += fm;
  };
  if (leaf) {
    for (int32_t s = lane; s < c; s += 32) source(T.offset + s, false);
  } else {
    for (int side = 0; side < 2; ++side) {
      const int32_t ch = side == 0 ? T.cl : T.cr;
      if (ch <= 0) continue;
      const DNode &C = nodes[ch];
      if (C.count <= 0) continue;
      if (C.count <= kQuad) {
        for (int32_t s = lane; s < C.count; s += 32) source(C.offset + s, false);
      } else if (lane < kQuad) {
        source(n + int64_t(kQuad) * ch + lane, true);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, o);
    gy += __shfl_xor_sync(0xffffffffu, gy, o);
    gz += __shfl_xor_sync(0xffffffffu, gz, o);
    gt += __shfl_xor_sync(0xffffffffu, gt, o);
  }
  if (lane == 0) {
    xcbar[3 * int64_t(t) + 0] = gx;
    xcbar[3 * int64_t(t) + 1] = gy;
    xcbar[3 * int64_t(t) + 2] = gz;
    tdrbar[t] = gt;
  }
}

// A block per node: tdr = ppc (x_max,d - xc_d) or ppc (xc_d - x_min,d), the
// face pptdr takes (its float expression, ties to the earlier face); the
// cotangent goes to the first particle of the node on that face and to xc.
__global__ void k_quad_adj_tdr(const DNode *__restrict__ nodes, int32_t nnodes,
                               const float4 *__restrict__ table, float ppc, float *xbx, float *xby,
                               float *xbz, float *xcbar, const float *tdrbar) {
  __shared__ int32_t best;
  const int32_t t = blockIdx.x;
  if (t >= nnodes) return;
  const float tb = tdrbar[t];
  const DNode &T = nodes[t];
  if (tb == 0.f || T.count <= 0) return;
  float cand[6];
  for (int d = 0; d < 3; ++d) {
    cand[d] = fsub_(T.xmax[d], T.xc[d]);
    cand[3 + d] = fsub_(T.xc[d], T.xmin[d]);
  }
  const float v = smin_(cand[0], smin_(cand[1], smin_(cand[2], smin_(cand[3],
                                                                   smin_(cand[4], cand[5])))));
  int face = 5;
  for (int j = 5; j >= 0; --j)
    if (cand[j] == v) face = j;
  const int d = face % 3;
  const float target = face < 3 ? T.xmax[d] : T.xmin[d];
  if (threadIdx.x == 0) best = INT32_MAX;
  __syncthreads();
  for (int32_t i = threadIdx.x; i < T.count; i += blockDim.x) {
    const float4 p = table[T.offset + i];
    const float x = d == 0 ? p.x : (d == 1 ? p.y : p.z);
    if (x == target) atomicMin(&best, i);
  }
  __syncthreads();
  if (threadIdx.x != 0 || best == INT32_MAX) return;
  const float g = ppc * tb;
  const int64_t k = T.offset + best;
  float *xb = d == 0 ? xbx : (d == 1 ? xby : xbz);
  atomicAdd(xb + k, face < 3 ? g : -g);
  xcbar[3 * int64_t(t) + d] += face < 3 ? -g : g;
}

// A warp per leaf: xbar_k += m_k sum over the nodes P on the leaf's
// root-to-leaf path of xcbar_P / M_P, M_P the node's mass (the sum of its
// points' masses, which is the sum of its particles' masses).
__global__ void k_quad_adj_paths(const DNode *__restrict__ nodes, int32_t nnodes,
                                 const float4 *__restrict__ table, int64_t n, float *xbx,
                                 float *xby, float *xbz, const float *xcbar, int32_t *err) {
  const int32_t leaf = int32_t((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (leaf >= nnodes) return;  // whole warps
  const DNode &L = nodes[leaf];
  if (L.cl != 0 || L.cr != 0 || L.count <= 0) return;
  const int32_t lo = L.offset;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f;
  int32_t t = 0;
  for (int depth = 0;; ++depth) {
    const float b0 = xcbar[3 * int64_t(t)], b1 = xcbar[3 * int64_t(t) + 1],
                b2 = xcbar[3 * int64_t(t) + 2];
    if (b0 != 0.f || b1 != 0.f || b2 != 0.f) {
      // the node's mass: lane a < 12 reads point a, summed over the warp
      float m = lane < kQuad ? table[n + int64_t(kQuad) * t + lane].w : 0.f;
      for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
      if (m != 0.f) {
        a0 += b0 / m;
        a1 += b1 / m;
        a2 += b2 / m;
      }
    }
    if (t == leaf) break;
    const DNode &T = nodes[t];
    const int32_t c = lo < T.offset + T.nleft ? T.cl : T.cr;
    if (c <= 0 || c >= nnodes || depth > 256) {  // cannot happen in a valid tree
      if (lane == 0) atomicExch(err, 5);
      return;
    }
    t = c;
  }
  if (a0 == 0.f && a1 == 0.f && a2 == 0.f) return;
  for (int32_t i = lane; i < L.count; i += 32) {
    const int32_t k = L.offset + i;
    const float m = table[k].w;
    xbx[k] += m * a0;
    xby[k] += m * a1;
    xbz[k] += m * a2;
  }
}

__global__ void k_iota(int32_t *p, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    p[i] = int32_t(i);
}

__global__ void k_fill_i64(int64_t *p, int64_t n, int64_t v) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    p[i] = v;
}

__global__ void k_root(DNode *nodes, int64_t n, TreeConfig cfg) {
  DNode &R = nodes[0];
  R.count = int32_t(n);
  R.offset = 0;
  R.cl = R.cr = 0;
  for (int d = 0; d < 3; ++d) {
    R.xmin[d] = cfg.min[d];
    R.xmax[d] = cfg.max[d];
    R.xc[d] = 0.f;
  }
  R.tdr = 0.f;
  R.split_dim = -1;
  R.nleft = 0;
}

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 0) {
  if (cap <= 0) cap = int64_t(sm_count()) * 32;
  int64_t b = (n + threads - 1) / threads;
  return unsigned(std::max<int64_t>(1, std::min(b, cap)));
}

}  // namespace

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------

// Deep levels (nodes of ~2048 elements or fewer on average): the chunk
// kernels run a warp per chunk.
inline bool wm_level(int64_t L, int64_t n) { return L * 2048 >= n; }

DeviceTree::~DeviceTree() {
  void *ptrs[] = {epos_, tpos_, oid_, toid_, idx_, nodes_, ppm_, chunk_node_, chunk_base_, part_,
                  left_cnt_, left_base_, scan_tmp_, node_tmp_, fallback_, counters_, leaf_ids_,
                  leaf_tmp_, leafdesc_, segs_, idx_list_, table_, items_, items_tmp_, gidx_,
                  tight_chunks_, tight_nodes_, segs_local_, ridx_, sub_nodes_, sub_first_,
                  sub_hist_, sub_pos_, sub_tot_, sub_stats_, wpre_, chains_};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h_counters_) cudaFreeHost(h_counters_);
  if (h_sub_) cudaFreeHost(h_sub_);
  if (aux_) {
    cudaStreamSynchronize(aux_);
    cudaStreamDestroy(aux_);
  }
  if (ev_fork_) cudaEventDestroy(ev_fork_);
  if (ev_groups_) cudaEventDestroy(ev_groups_);
}

template <typename T>
cudaError_t DeviceTree::grow(T *&p, size_t &cap, size_t count, cudaStream_t s, bool keep) {
  if (count <= cap && p) return cudaSuccess;
  size_t want = std::max<size_t>(count + count / 4, 256);
  T *q = nullptr;
  cudaError_t e = cudaMalloc(&q, want * sizeof(T));
  if (e != cudaSuccess) return e;
  if (keep && p && cap) {
    e = cudaMemcpyAsync(q, p, cap * sizeof(T), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
  }
  if (p) cudaFree(p);
  p = q;
  cap = want;
  return cudaSuccess;
}

#define DT_CHECK(x)                         \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return e_;       \
  } while (0)

cudaError_t DeviceTree::build(const TreeConfig &cfg, int64_t n, const float4 *pos_in, int64_t jsplit,
                              cudaStream_t s) {
  info_ = DeviceTreeInfo{};
  err_ = nullptr;
  padded_pairs_ = 0;
  if (aux_) {  // a previous build that stopped early may have left its groups running
    DT_CHECK(cudaStreamSynchronize(aux_));
    groups_ready_ = 0;
  }
  const auto t0 = std::chrono::steady_clock::now();
  const int k = cfg.tdpts;
  const size_t nn = size_t(std::max<int64_t>(n, 1));
  n_ = n;
  DT_CHECK(grow(tight_chunks_, cap_tc_,
                (size_t(n) / kTightChunk + kTightNodes + 1) * (sizeof(TightChunk) / sizeof(double)), s));
  DT_CHECK(grow(tight_nodes_, cap_tn_, size_t(kTightNodes) * (sizeof(TightNode) / sizeof(double)), s));
  DT_CHECK(grow(epos_, cap_e_, nn, s));
  DT_CHECK(grow(tpos_, cap_t_, nn, s));
  DT_CHECK(grow(oid_, cap_o_, nn, s));
  DT_CHECK(grow(toid_, cap_to_, nn, s));
  DT_CHECK(grow(idx_, cap_i_, nn, s));
  DT_CHECK(grow(ridx_, cap_ri_, nn, s));
  if (!counters_) {
    DT_CHECK(cudaMalloc(&counters_, C_COUNT * sizeof(int64_t)));
    DT_CHECK(cudaHostAlloc(&h_counters_, C_COUNT * sizeof(int64_t), cudaHostAllocDefault));
    // the kernels' error flag lives in a counter slot: read back with the counters
    walk_err_ = reinterpret_cast<int32_t *>(counters_ + C_ERR);
  }
  DT_CHECK(cudaMemsetAsync(counters_, 0, C_COUNT * sizeof(int64_t), s));
  if (n > 0) {
    DT_CHECK(cudaMemcpyAsync(epos_, pos_in, size_t(n) * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(oid_, n);
    ++info_.launches;
  }
  size_t want_nodes = size_t(std::max<int64_t>(64, 4 * n / std::max(1, cfg.nd) + 64));
  DT_CHECK(grow(nodes_, cap_nodes_, want_nodes, s));
  k_root<<<1, 1, 0, s>>>(nodes_, n, cfg);
  ++info_.launches;
  DT_CHECK(cudaGetLastError());

  // ---- levels ----
  std::vector<int32_t> level_begin{0};
  int32_t nb = 0, ne = 1;
  int64_t level_max = n;  // the level's largest node
  if (!node_attr_) {
    DT_CHECK(cudaFuncSetAttribute(k_part_node<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kNodeMax * int(sizeof(int32_t))));
    DT_CHECK(cudaFuncSetAttribute(k_part_node<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kNodeMax * int(sizeof(int32_t))));
    node_attr_ = true;
  }
  while (ne > nb) {
    const int32_t L = ne - nb;
    if (!sub_off_ && cfg.force_cm_fallback != 2 && level_max <= kSubMax) {
      // every node of this level fits one block: each builds its whole subtree
      DT_CHECK(grow(sub_nodes_, cap_sub_, size_t(2 * std::max<int64_t>(n, 1)), s));
      DT_CHECK(grow(sub_stats_, cap_ss_, size_t(std::max<int64_t>(n, 1)) * sizeof(SubWarpStats), s));
      DT_CHECK(grow(sub_first_, cap_sf_, size_t(L) * (kSubDepth + 2), s));
      DT_CHECK(grow(sub_hist_, cap_sh_, size_t(L) * kSubDepth + 1, s));
      DT_CHECK(grow(sub_pos_, cap_sp_, size_t(L) * kSubDepth + 1, s));
      DT_CHECK(grow(sub_tot_, cap_st_, size_t(kSubDepth), s));
      DT_CHECK(grow(scan_tmp_, cap_scan_, size_t(scan_tmp_size(int64_t(L) * kSubDepth)), s));
      if (!h_sub_) DT_CHECK(cudaHostAlloc(&h_sub_, kSubDepth * sizeof(int64_t), cudaHostAllocDefault));
      if (!sub_attr_) {
        DT_CHECK(cudaFuncSetAttribute(k_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kSubMax * int(sizeof(int32_t))));
        sub_attr_ = true;
      }
      const size_t smem = size_t(std::max<int64_t>(level_max, 1)) * sizeof(int32_t);
      k_subtree<<<unsigned(L), kSubThreads, smem, s>>>(
          nodes_, nb, ne, epos_, oid_, tpos_, toid_, sub_nodes_,
          reinterpret_cast<SubWarpStats *>(sub_stats_), sub_first_, sub_hist_,
          cfg.force_cm_fallback, cfg.nd, counters_);
      ++info_.launches;
      DT_CHECK(cudaGetLastError());
      DT_CHECK(scan_counted(sub_hist_, sub_pos_, int64_t(L) * kSubDepth, nullptr, scan_tmp_, s));
      k_subtree_totals<<<kSubDepth, 256, 0, s>>>(sub_hist_, L, sub_tot_);
      ++info_.launches;
      DT_CHECK(cudaGetLastError());
      DT_CHECK(cudaMemcpyAsync(h_sub_, sub_tot_, kSubDepth * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
      DT_CHECK(cudaMemcpyAsync(h_counters_, counters_, C_COUNT * sizeof(int64_t),
                               cudaMemcpyDeviceToHost, s));
      DT_CHECK(cudaStreamSynchronize(s));
      const int32_t serr = *reinterpret_cast<const int32_t *>(h_counters_ + C_ERR);
      if (serr == 4) {
        // a subtree deeper than kSubDepth levels: build again level by level
        sub_off_ = true;
        const cudaError_t e = build(cfg, n, pos_in, jsplit, s);
        sub_off_ = false;
        return e;
      }
      if (serr) {
        err_ = serr == 3 ? "subtree: a node outgrew the block's shared memory"
                         : "partition chain check failed";
        return cudaErrorUnknown;
      }
      info_.cm_fallbacks += h_counters_[C_SUBFB];
      int64_t total = ne;
      for (int d = 0; d < kSubDepth; ++d) total += h_sub_[d];
      if (total > INT32_MAX) return cudaErrorInvalidValue;
      DT_CHECK(grow(nodes_, cap_nodes_, size_t(total), s, true));
      k_subtree_place<<<unsigned(L), 256, 0, s>>>(nodes_, nb, ne, sub_nodes_, sub_first_, sub_pos_);
      ++info_.launches;
      DT_CHECK(cudaGetLastError());
      int64_t at = ne;
      level_begin.push_back(ne);
      for (int d = 0; d < kSubDepth && h_sub_[d] > 0; ++d) {
        at += h_sub_[d];
        level_begin.push_back(int32_t(at));
      }
      nb = ne = int32_t(total);
      break;
    }
    if (size_t(ne) + 2 * size_t(L) > cap_nodes_)
      DT_CHECK(grow(nodes_, cap_nodes_, size_t(ne) + 2 * size_t(L), s, true));
    DT_CHECK(grow(node_tmp_, cap_nt_, size_t(L) + 1, s));
    DT_CHECK(grow(chunk_base_, cap_cb_, size_t(L) + 1, s));
    DT_CHECK(grow(scan_tmp_, cap_scan_, size_t(scan_tmp_size(std::max<int64_t>(L, n + 1))), s));
    DT_CHECK(grow(fallback_, cap_fb_, size_t(L), s));
    const int64_t max_chunks = n / kChunk + L + 1;
    DT_CHECK(grow(chunk_node_, cap_cn_, size_t(max_chunks), s));
    DT_CHECK(grow(part_, cap_part_, size_t(max_chunks) * kPartWords, s));
    DT_CHECK(grow(left_cnt_, cap_lc_, size_t(max_chunks), s));
    DT_CHECK(grow(left_base_, cap_lb_, size_t(max_chunks), s));
    DT_CHECK(grow(wpre_, cap_wp_, size_t(max_chunks) * (kChunkThreads / 32), s));
    if (level_max > kNodeMax && !wm_level(L, n))
      DT_CHECK(grow(chains_, cap_ch_, size_t(std::max<int64_t>(n, 1)), s));
    const unsigned gL = unsigned((L + 127) / 128);
    const bool small = int64_t(L) <= kScanBlock;
    if (small) {
      k_chunk_setup_small<<<1, kScanThreads, 0, s>>>(nodes_, nb, ne, chunk_base_, chunk_node_,
                                                     counters_);
      ++info_.launches;
    } else {
      DT_CHECK(cudaMemsetAsync(counters_ + C_NFALLBACK, 0, sizeof(int64_t), s));
      DT_CHECK(cudaMemsetAsync(counters_ + C_NTIGHT, 0, sizeof(int64_t), s));
      DT_CHECK(cudaMemsetAsync(counters_ + C_MAXCNT, 0, sizeof(int64_t), s));
      DT_CHECK(cudaMemsetAsync(counters_ + C_CHAINS, 0, sizeof(int64_t), s));
      k_chunk_counts<<<gL, 128, 0, s>>>(nodes_, nb, ne, node_tmp_);
      ++info_.launches;
      DT_CHECK(scan_counted(node_tmp_, chunk_base_, L, counters_ + C_NCHUNK, scan_tmp_, s));
      k_chunk_fill<<<gL, 128, 0, s>>>(nodes_, nb, ne, chunk_base_, chunk_node_);
      ++info_.launches;
    }
    // deep levels (nodes of ~2048 elements or fewer on average): a warp per chunk
    const bool wm = wm_level(L, n);
    const unsigned gC = wm ? unsigned((max_chunks + 7) / 8) : unsigned(max_chunks);
#define CHUNK_LAUNCH(kern, ...)                                                  \
  do {                                                                           \
    if (wm) kern<true><<<gC, kChunkThreads, 0, s>>>(__VA_ARGS__);                \
    else kern<false><<<gC, kChunkThreads, 0, s>>>(__VA_ARGS__);                  \
    ++info_.launches;                                                            \
  } while (0)
    CHUNK_LAUNCH(k_stats_partial, epos_, nodes_, chunk_node_, chunk_base_, nb, counters_ + C_NCHUNK,
                 part_);
    // one thread finishes each single-chunk node, a warp each larger one; a
    // small level with larger nodes has a warp finish every node in one launch
    const bool one_chunk = level_max <= kChunk;
    const bool big_nodes = L <= 16 && level_max > 32 * int64_t(kChunk);
    if (big_nodes) {
      // the top levels: a block per node (every node of the level)
      k_stats_final_block<<<unsigned(L), 256, 0, s>>>(nodes_, nb, ne, chunk_base_, part_, fallback_,
                                                      counters_, cfg.force_cm_fallback, cfg.nd);
      ++info_.launches;
    } else if (!small || one_chunk) {
      k_stats_final_one<<<gL, 128, 0, s>>>(nodes_, nb, ne, chunk_base_, part_, fallback_,
                                            counters_, cfg.force_cm_fallback, cfg.nd);
      ++info_.launches;
    }
    if (!one_chunk && !big_nodes) {
      k_stats_final<<<unsigned((int64_t(L) * 32 + 255) / 256), 256, 0, s>>>(
          nodes_, nb, ne, chunk_base_, part_, fallback_, counters_, cfg.force_cm_fallback, cfg.nd,
          small);
      ++info_.launches;
    }
    k_cm_tight_sums<<<tight_blocks(), kTightThreads, 0, s>>>(
        epos_, nodes_, fallback_, counters_, reinterpret_cast<TightChunk *>(tight_chunks_),
        reinterpret_cast<TightNode *>(tight_nodes_), cfg.force_cm_fallback == 1);
    ++info_.launches;
    k_cm_tight_bound<<<tight_blocks(), kTightThreads, 0, s>>>(
        epos_, nodes_, fallback_, counters_, reinterpret_cast<const TightChunk *>(tight_chunks_),
        reinterpret_cast<TightNode *>(tight_nodes_), cfg.force_cm_fallback == 1);
    ++info_.launches;
    k_cm_fallback<<<unsigned(std::min<int64_t>((L + 127) / 128, 1024)), 128, 0, s>>>(
        epos_, nodes_, fallback_, counters_);
    ++info_.launches;
    if (level_max <= kNodeMax) {
      // every node fits one block's shared memory: the whole partition in one launch
      const size_t smem = size_t(std::max<int64_t>(level_max, 1)) * sizeof(int32_t);
      // few large nodes: 1024 threads a node; many (most of them small, as in
      // clustered sets): 256
      if (level_max > 2048 && L <= 1024)
        k_part_node<1024><<<unsigned(L), 1024, smem, s>>>(epos_, oid_, nodes_, nb, ne,
                                                          int32_t(level_max), tpos_, toid_, walk_err_);
      else
        k_part_node<256><<<unsigned(L), 256, smem, s>>>(epos_, oid_, nodes_, nb, ne,
                                                        int32_t(level_max), tpos_, toid_, walk_err_);
      ++info_.launches;
    } else {
      CHUNK_LAUNCH(k_part_count, epos_, nodes_, chunk_node_, chunk_base_, nb, counters_ + C_NCHUNK,
                   left_cnt_, wpre_);
      k_part_node_scan<<<unsigned((int64_t(L) * 32 + 127) / 128), 128, 0, s>>>(
          nodes_, nb, ne, chunk_base_, left_cnt_, left_base_);
      ++info_.launches;
      CHUNK_LAUNCH(k_part_left, epos_, oid_, nodes_, chunk_node_, chunk_base_, nb,
                   counters_ + C_NCHUNK, left_base_, wpre_, tpos_, toid_, idx_, ridx_);
      CHUNK_LAUNCH(k_part_right, epos_, oid_, nodes_, chunk_node_, chunk_base_, nb,
                   counters_ + C_NCHUNK, idx_, ridx_, tpos_, toid_, walk_err_, counters_,
                   reinterpret_cast<ChainItem *>(chains_), int64_t(cap_ch_));
      if (!wm) {
        k_part_chains<<<unsigned(4 * sm_count()), 256, 0, s>>>(
            epos_, oid_, nodes_, reinterpret_cast<const ChainItem *>(chains_), int64_t(cap_ch_),
            counters_, idx_, ridx_, tpos_, toid_, walk_err_);
        ++info_.launches;
      }
    }
#undef CHUNK_LAUNCH
    std::swap(epos_, tpos_);
    std::swap(cap_e_, cap_t_);
    std::swap(oid_, toid_);
    std::swap(cap_o_, cap_to_);
    // one block sets up the children of a level of up to 1024 nodes; above
    // that its stores alone take longer than the three-kernel path
    if (L <= 1024) {
      k_children_small<<<1, kScanThreads, 0, s>>>(nodes_, nb, ne, counters_ + C_NSPLIT,
                                                  counters_ + C_MAXCNT);
      ++info_.launches;
    } else {
      k_split_flags<<<gL, 128, 0, s>>>(nodes_, nb, ne, node_tmp_);
      ++info_.launches;
      DT_CHECK(scan_counted(node_tmp_, node_tmp_, L, counters_ + C_NSPLIT, scan_tmp_, s));
      k_children<<<gL, 128, 0, s>>>(nodes_, nb, ne, node_tmp_, counters_ + C_MAXCNT);
      ++info_.launches;
    }
    DT_CHECK(cudaGetLastError());
    DT_CHECK(cudaMemcpyAsync(h_counters_, counters_, (C_ERR + 1) * sizeof(int64_t),
                             cudaMemcpyDeviceToHost, s));
    DT_CHECK(cudaStreamSynchronize(s));
    const int32_t perr = *reinterpret_cast<const int32_t *>(h_counters_ + C_ERR);
    if (perr) {
      err_ = perr == 3 ? "partition: a node outgrew the one-block partition's shared memory"
                       : "partition chain check failed";
      return cudaErrorUnknown;
    }
    info_.cm_fallbacks += h_counters_[C_NFALLBACK] - h_counters_[C_NTIGHT];
    const int64_t nsplit = h_counters_[C_NSPLIT];
    level_max = h_counters_[C_MAXCNT];
    nb = ne;
    ne = int32_t(ne + 2 * nsplit);
    level_begin.push_back(nb);
  }
  levels_ = level_begin;
  const int32_t nnodes = ne;
  info_.nodes = nnodes;
  const auto t1 = std::chrono::steady_clock::now();
  build_ms_ = std::chrono::duration<double, std::milli>(t1 - t0).count();
  info_.levels = int64_t(level_begin.size()) - 1;

  // ---- pseudo-particles, deepest level first ----
  DT_CHECK(grow(ppm_, cap_ppm_, size_t(nnodes) * k + 1, s));
  {
    // the top levels of at most 1024 nodes each in one launch, the rest a
    // launch per level
    const int64_t nlev = int64_t(level_begin.size()) - 1;
    int64_t lt = 0;
    while (lt < nlev && lt < kTopLevels && level_begin[lt + 1] - level_begin[lt] <= 1024) ++lt;
    for (int64_t l = nlev - 1; l >= lt; --l) {
      const int32_t lb = level_begin[l], le = level_begin[l + 1];
      if (le > lb) {
        k_pseudo<<<unsigned((int64_t(le - lb) * 32 + 255) / 256), 256, 0, s>>>(
            nodes_, lb, le, epos_, ppm_, k, cfg.ppc, cfg.nd);
        ++info_.launches;
      }
    }
    if (lt > 0) {
      LevelSpan lv{};
      lv.n = int32_t(lt);
      for (int64_t l = 0; l <= lt; ++l) lv.b[l] = level_begin[l];
      k_pseudo_top<<<1, 1024, 0, s>>>(nodes_, lv, epos_, ppm_, k, cfg.ppc, cfg.nd);
      ++info_.launches;
    }
  }
  const int64_t ntab = n + int64_t(nnodes) * k;
  DT_CHECK(grow(table_, cap_tab_, size_t(std::max<int64_t>(ntab, 1)), s));
  if (n > 0)
    DT_CHECK(cudaMemcpyAsync(table_, epos_, size_t(n) * sizeof(float4), cudaMemcpyDeviceToDevice, s));
  k_table_pseudo<<<unsigned((nnodes + 127) / 128), 128, 0, s>>>(nodes_, nnodes, ppm_, k, table_, n);
  ++info_.launches;
  DT_CHECK(cudaGetLastError());

  // ---- processed leaves in DFS order ----
  const int64_t nl_cap = std::max<int64_t>(n, 1);
  DT_CHECK(grow(leaf_tmp_, cap_lt_, size_t(2 * nl_cap), s));
  DT_CHECK(grow(leaf_ids_, cap_leaf_, size_t(nl_cap), s));
  DT_CHECK(grow(scan_tmp_, cap_scan_, size_t(scan_tmp_size(nl_cap)), s));
  int64_t *leaf_at = leaf_tmp_, *lflag = leaf_tmp_ + nl_cap;
  k_fill_i64<<<grid_for(nl_cap, 256), 256, 0, s>>>(leaf_at, nl_cap, -1);
  ++info_.launches;
  k_mark_leaves<<<unsigned((nnodes + 127) / 128), 128, 0, s>>>(nodes_, nnodes, cfg, n, leaf_at);
  ++info_.launches;
  k_leaf_flags<<<unsigned((nl_cap + 255) / 256), 256, 0, s>>>(leaf_at, nl_cap, lflag);
  ++info_.launches;
  DT_CHECK(scan_counted(lflag, lflag, nl_cap, counters_ + C_NLEAF, scan_tmp_, s));
  k_leaf_compact<<<unsigned((nl_cap + 255) / 256), 256, 0, s>>>(leaf_at, lflag, nl_cap, leaf_ids_);
  ++info_.launches;
  DT_CHECK(cudaGetLastError());
  DT_CHECK(cudaMemcpyAsync(h_counters_ + C_NLEAF, counters_ + C_NLEAF, sizeof(int64_t),
                           cudaMemcpyDeviceToHost, s));
  DT_CHECK(cudaStreamSynchronize(s));
  const int64_t nleaves = h_counters_[C_NLEAF];
  info_.processed_leaves = nleaves;
  // the groups need only the leaves: on the second stream, beside the walk
  // (forked here, launched after the walk)
  group_ = cfg.group == 16 ? 16 : 32;
  DT_CHECK(grow(gidx_, cap_gidx_, size_t(std::max<int64_t>(n, 1)), s));
  if (nleaves > 0) {
    if (!aux_) {
      DT_CHECK(cudaStreamCreateWithFlags(&aux_, cudaStreamNonBlocking));
      DT_CHECK(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
      DT_CHECK(cudaEventCreateWithFlags(&ev_groups_, cudaEventDisableTiming));
    }
    DT_CHECK(cudaEventRecord(ev_fork_, s));
    DT_CHECK(cudaStreamWaitEvent(aux_, ev_fork_, 0));
  }

  // ---- lists: count, scan, write ----
  const size_t nlw = size_t(std::max<int64_t>(nleaves, 1));
  DT_CHECK(grow(node_tmp_, cap_nt_, 5 * nlw + 4, s));
  int64_t *seg_cnt = node_tmp_, *list_len = node_tmp_ + nlw, *seg_base = node_tmp_ + 2 * nlw,
          *list_base = node_tmp_ + 3 * nlw;
  DT_CHECK(grow(scan_tmp_, cap_scan_, size_t(scan_tmp_size(int64_t(nlw))), s));
  // one pass writing each leaf's segments into its own region; the scans
  // then place them (a leaf with more than kLocalSegs segments sends the
  // build to a second, placing walk)
  DT_CHECK(grow(segs_local_, cap_segl_, nlw * kLocalSegs, s));
  DT_CHECK(cudaMemsetAsync(counters_ + C_SEGOVF, 0, sizeof(int64_t), s));
  if (nleaves > 0) {
    k_walk<2><<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(
        nodes_, nnodes, leaf_ids_, nleaves, cfg, n, seg_cnt, list_len, nullptr, nullptr,
        segs_local_, walk_err_, counters_);
    ++info_.launches;
    // the groups after the walk's blocks, which then have their SMs first
    DT_CHECK(launch_groups(nleaves, group_, aux_));
    DT_CHECK(cudaEventRecord(ev_groups_, aux_));
    groups_ready_ = group_;
    DT_CHECK(scan_counted(seg_cnt, seg_base, nleaves, counters_ + C_NSEG, scan_tmp_, s));
    DT_CHECK(scan_counted(list_len, list_base, nleaves, counters_ + C_NENT, scan_tmp_, s));
  }
  DT_CHECK(cudaGetLastError());
  // segments, entries, the overflow flag and the error flag in one copy
  DT_CHECK(cudaMemcpyAsync(h_counters_ + C_NSEG, counters_ + C_NSEG,
                           (C_ERR + 1 - C_NSEG) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  DT_CHECK(cudaStreamSynchronize(s));
  const int32_t h_err = *reinterpret_cast<const int32_t *>(h_counters_ + C_ERR);
  if (h_err) {
    err_ = h_err == 1 ? "interaction-list walk exceeded its stack"
                      : "interaction-list walk visited more nodes than the tree has";
    return cudaErrorUnknown;
  }
  const int64_t nseg = nleaves > 0 ? h_counters_[C_NSEG] : 0;
  const int64_t nent = nleaves > 0 ? h_counters_[C_NENT] : 0;
  info_.segments = nseg;
  info_.list_entries = nent;
  DT_CHECK(grow(segs_, cap_seg_, size_t(std::max<int64_t>(nseg, 1)), s));
  DT_CHECK(grow(idx_list_, cap_idx_, size_t(std::max<int64_t>(nent, 1)), s));
  DT_CHECK(grow(leafdesc_, cap_ld_, nlw, s));
  if (nleaves > 0) {
    if (h_counters_[C_SEGOVF]) {
      k_walk<1><<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(
          nodes_, nnodes, leaf_ids_, nleaves, cfg, n, nullptr, nullptr, seg_base, list_base, segs_,
          walk_err_, counters_);
      ++info_.launches;
    } else {
      k_pack_segs<<<unsigned(std::min<int64_t>((nleaves + 7) / 8, int64_t(sm_count()) * 64)), 256, 0, s>>>(
          segs_local_, seg_cnt, seg_base, list_base, nleaves, segs_);
      ++info_.launches;
    }
    int64_t *kept = nullptr;
    if (cfg.prune2 > 0.0f) {
      kept = node_tmp_ + 4 * nlw;
      int64_t blocks = std::min<int64_t>((nleaves + 7) / 8, int64_t(sm_count()) * 64);
      k_expand_pruned<<<unsigned(blocks), 256, 0, s>>>(segs_, seg_base, seg_cnt, list_base, nodes_,
                                                       leaf_ids_, nleaves, table_, cfg.prune2,
                                                       idx_list_, kept);
      ++info_.launches;
    } else {
      DT_CHECK(launch_expand_segments(segs_, nseg, idx_list_, s));
      info_.launches += nseg > 0;
    }
    k_leaf_desc<<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(
        nodes_, leaf_ids_, nleaves, list_len, kept, list_base, leafdesc_, counters_);
    ++info_.launches;
  }
  DT_CHECK(cudaGetLastError());

  // ---- work items ----
  DT_CHECK(make_items(n, jsplit, s));
  lists_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
  return cudaSuccess;
}

cudaError_t DeviceTree::scan_counted(const int64_t *in, int64_t *out, int64_t n, int64_t *total,
                                     int64_t *tmp, cudaStream_t s) {
  // one block-scan launch per level of the recursion plus one add per level above the last
  for (int64_t m = n; m > 0;) {
    ++info_.launches;
    const int64_t nb = (m + kScanBlock - 1) / kScanBlock;
    if (nb == 1) break;
    ++info_.launches;
    m = nb;
  }
  return exclusive_scan_i64(in, out, n, total, tmp, s);
}

cudaError_t DeviceTree::regroup(int group, int64_t jsplit, cudaStream_t s) {
  if (group != 16 && group != 32) return cudaErrorInvalidValue;
  group_ = group;
  return make_items(n_, jsplit, s);
}

cudaError_t DeviceTree::launch_groups(int64_t nleaves, int G, cudaStream_t s) {
  k_groups_warp<<<unsigned((nleaves + kGWarps - 1) / kGWarps), 32 * kGWarps, 0, s>>>(
      nodes_, leaf_ids_, nleaves, epos_, gidx_, G);
  k_groups<<<unsigned(nleaves), kGroupThreads, 0, s>>>(nodes_, leaf_ids_, nleaves, epos_, gidx_, G);
  info_.launches += 2;
  return cudaGetLastError();
}

cudaError_t DeviceTree::make_items(int64_t n, int64_t jsplit, cudaStream_t s) {
  const int64_t nleaves = info_.processed_leaves;
  const int G = group_;
  DT_CHECK(grow(gidx_, cap_gidx_, size_t(std::max<int64_t>(n, 1)), s));
  DT_CHECK(cudaMemsetAsync(counters_ + C_BUCKET, 0, 32 * sizeof(int64_t), s));
  if (nleaves > 0) {
    if (groups_ready_ == G) {
      DT_CHECK(cudaStreamWaitEvent(s, ev_groups_, 0));  // launched by build()
    } else {
      if (groups_ready_) DT_CHECK(cudaStreamWaitEvent(s, ev_groups_, 0));
      DT_CHECK(launch_groups(nleaves, G, s));
    }
    groups_ready_ = 0;
    k_item_hist<<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(leafdesc_, nleaves, jsplit, G,
                                                                counters_);
    ++info_.launches;
    k_item_bases<<<1, 32, 0, s>>>(counters_);
    ++info_.launches;
  }
  DT_CHECK(cudaGetLastError());
  DT_CHECK(cudaMemcpyAsync(h_counters_, counters_, C_COUNT * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  DT_CHECK(cudaStreamSynchronize(s));
  const int64_t nitems = nleaves > 0 ? h_counters_[C_NITEMS] : 0;
  info_.items = nitems;
  info_.pairs = h_counters_[C_PAIRS];
  padded_pairs_ = h_counters_[C_PADDED];
  DT_CHECK(grow(items_, cap_items_, size_t(std::max<int64_t>(nitems, 1)), s));
  if (nitems > 0) {
    k_item_fill<<<unsigned((nleaves + 127) / 128), 128, 0, s>>>(leafdesc_, nleaves, jsplit, G,
                                                               counters_, items_);
    ++info_.launches;
  }
  DT_CHECK(cudaGetLastError());
  DT_CHECK(cudaStreamSynchronize(s));
  return cudaSuccess;
}

cudaError_t launch_gather_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_gather<float><<<grid_for(n, 256), 256, 0, s>>>(in, perm, out, n);
  return cudaGetLastError();
}
cudaError_t launch_gather3_f32(const float *a, const float *b, const float *c, const int32_t *perm,
                               float *out, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_gather3_f32<<<grid_for(n, 256), 256, 0, s>>>(a, b, c, perm, out, n);
  return cudaGetLastError();
}
cudaError_t launch_outputs(const float4 *table, const float *phi, const int64_t *id,
                           const uint16_t *mask, const int32_t *perm, float *x, float *y, float *z,
                           float *m, float *ophi, int64_t *oid, uint16_t *omask, int64_t n,
                           cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_outputs<<<grid_for(n, 256), 256, 0, s>>>(table, phi, id, mask, perm, x, y, z, m, ophi, oid,
                                             omask, n);
  return cudaGetLastError();
}
cudaError_t launch_scatter_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                               cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_scatter_f32<<<grid_for(n, 256), 256, 0, s>>>(in, perm, out, n);
  return cudaGetLastError();
}

cudaError_t launch_scatter_add_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                                   cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_scatter_add_f32<<<grid_for(n, 256), 256, 0, s>>>(in, perm, out, n);
  return cudaGetLastError();
}

cudaError_t launch_pseudo_adjoint(const DNode *nodes, const std::vector<int32_t> &levels,
                                  const float4 *table, int64_t n, float *xbx, float *xby,
                                  float *xbz, int32_t *err, cudaStream_t s) {
  if (levels.size() < 2) return cudaSuccess;
  const int32_t nnodes = levels.back();
  if (nnodes <= 0) return cudaSuccess;
  k_adj_paths<<<unsigned((int64_t(nnodes) * 32 + 255) / 256), 256, 0, s>>>(nodes, nnodes, table, n,
                                                                           xbx, xby, xbz, err);
  return cudaGetLastError();
}

cudaError_t launch_pseudo_adjoint_quad(const DNode *nodes, const std::vector<int32_t> &levels,
                                       const float4 *table, int64_t n, int32_t nd, float ppc,
                                       float *xbx, float *xby, float *xbz, float *mb, float *xcbar,
                                       float *tdrbar, int32_t *err, cudaStream_t s) {
  if (levels.size() < 2) return cudaSuccess;
  const int32_t nnodes = levels.back();
  if (nnodes <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(xcbar, 0, size_t(nnodes) * 3 * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(tdrbar, 0, size_t(nnodes) * sizeof(float), s);
  if (e != cudaSuccess) return e;
  for (size_t l = 0; l + 1 < levels.size(); ++l) {
    const int32_t lb = levels[l], le = levels[l + 1];
    if (le > lb)
      k_quad_adj_level<<<unsigned((int64_t(le - lb) * 32 + 255) / 256), 256, 0, s>>>(
          nodes, lb, le, table, n, nd, xbx, xby, xbz, mb, xcbar, tdrbar);
  }
  k_quad_adj_tdr<<<unsigned(nnodes), 256, 0, s>>>(nodes, nnodes, table, ppc, xbx, xby, xbz, xcbar,
                                                  tdrbar);
  k_quad_adj_paths<<<unsigned((int64_t(nnodes) * 32 + 255) / 256), 256, 0, s>>>(
      nodes, nnodes, table, n, xbx, xby, xbz, xcbar, err);
  return cudaGetLastError();
}

cudaError_t launch_pack4(const float *x, const float *y, const float *z, const float *m,
                         float4 *out, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_pack4<<<grid_for(n, 256), 256, 0, s>>>(x, y, z, m, out, n);
  return cudaGetLastError();
}
}  // namespace hsr
