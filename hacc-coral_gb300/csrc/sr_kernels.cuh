// sr_kernels.cuh -- device side of the short-range pair interaction.
//
// The pair term is the reference's nbody1 inner loop
// (src/halo_finder/RCBForceTree.cxx:599-619) with ForceLawSR over
// FGridEvalPoly (src/halo_finder/ForceLaw.cxx:137-141, 187-192):
//   g(r2) = (r2 + rsm^2)^(-3/2) - sum_{k=0..6} a_k r2^k,
//   a_i  += [r2 < fsrrmax^2] m_j g(r2) (x_j - x_i),   v_i += fcoeff m_i a_i.
// FP32 on the CUDA cores: (r2 + rsm^2)^(-3/2) is y^3 with y = rsqrt(r2 +
// rsm^2), and the polynomial is subtracted inside the final multiply-add
// (g = y * y^2 + (-p)), which is 20 FMA-pipe operations and one MUFU per pair.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hsr {

enum { LAW_POLY6 = 0, LAW_POLY5_STEP16 = 1 };

// Work description of one processed leaf on the device.
struct alignas(16) LeafDesc {
  int32_t offset;      // first particle of the leaf in the position table
  int32_t count;       // particles in the leaf
  int32_t list_len;    // entries in its interaction list (self included)
  int32_t kept_len;    // entries in the index array: the list less the entries
                       // farther than the cutoff from the leaf's box (they add
                       // exactly 0 to every particle of the leaf), or list_len
                       // where the list is not pruned
  int64_t list_begin;  // first entry of the list in the index array
  int64_t pad2;
};

// Segment of consecutive position-table entries, expanded into the index
// array at `dst`.
struct alignas(16) SegDesc {
  int32_t start;
  int32_t count;
  int64_t dst;
};

// Work item of the batched kernel: one group of at most 32 particles of a
// leaf (spatially compact, listed in the group index array at g_begin)
// against a contiguous range of that leaf's list.  Items of a group whose list
// is split over several items accumulate with atomics (flags & 1).
struct alignas(16) PairItem {
  int64_t j_begin;   // first entry in the index array
  int32_t j_len;     // entries in this item
  int32_t g_begin;   // first particle of the group in the group index array
  int32_t g_count;   // particles in the group (1..32)
  int32_t flags;     // bit 0: list split over several items
  int64_t pad;
};

// The law in terms of s = r2 + rsm^2, for the batched kernel: g = s^-3/2 +
// q(s) with q(s) = -p(s - rsm^2) re-expanded in s (nb[k], computed in double
// and rounded), and the cutoff as s < scut (scut = rcut2 + rsm^2 in float).
// Step16 also drops s <= rsm^2, i.e. r2 == 0.
struct LawS {
  float nb[7];
  float rsm2, scut;
  int32_t drop_self;
};

// One box of a multi-box launch: where its work lives and its kick
// parameters.  Items carry their box in flags >> 8.
struct alignas(16) BoxDesc {
  const float4 *table;
  const int32_t *idx;
  const int32_t *gidx;
  float *vx, *vy, *vz;
  float fcoeff, rsm2, rcut2, rcull2;
  LawS law;
};

// One box of a multi-box adjoint launch: its tape (table, lists, groups),
// the cotangent in tree order and the gradient table it adds into (particles,
// then pseudo-particle slots).  Items carry their box in flags >> 8.
struct alignas(16) VjpBoxDesc {
  const float4 *table;
  const int32_t *idx;
  const int32_t *gidx;
  const float *ux, *uy, *uz;
  float *xbx, *xby, *xbz;
  float fcoeff, rsm2, rcut2, rcull2;
  float *mb;      // 12-point boxes: the pseudo-particles' mass cotangents, else null
  int64_t npart;  // the box's particles (table entries below are not pseudo-particles)
};

// LawS of a law with softening rsm and strict cutoff rcut2 on r2.
LawS make_law_s(int law, float rsm2, float rcut2);

#if defined(__CUDACC__)
// -p(r2) for the law's polynomial, in Horner form on negated coefficients.
// The coefficients are the reference's double literals rounded to float, as
// FGridEvalPoly stores them in float m_a[7] (ForceLaw.cxx:98-104) and
// Step16_int writes them (BGQStep16.c:167).
template <int LAW>
__device__ __forceinline__ float neg_poly(float r2);

template <>
__device__ __forceinline__ float neg_poly<LAW_POLY6>(float r2) {
  float q = -static_cast<float>(0.000000147305);
  q = fmaf(q, r2, -static_cast<float>(-0.00000663394));
  q = fmaf(q, r2, -static_cast<float>(0.000132336));
  q = fmaf(q, r2, -static_cast<float>(-0.00159485));
  q = fmaf(q, r2, -static_cast<float>(0.0133122));
  q = fmaf(q, r2, -static_cast<float>(-0.0783394));
  q = fmaf(q, r2, -static_cast<float>(0.271431));
  return q;
}

template <>
__device__ __forceinline__ float neg_poly<LAW_POLY5_STEP16>(float r2) {
  float q = -static_cast<float>(-0.00000147177);
  q = fmaf(q, r2, -static_cast<float>(0.0000605491));
  q = fmaf(q, r2, -static_cast<float>(-0.00109313));
  q = fmaf(q, r2, -static_cast<float>(0.0114808));
  q = fmaf(q, r2, -static_cast<float>(-0.0750978));
  q = fmaf(q, r2, -static_cast<float>(0.269327));
  return q;
}

// g(r2) without the cutoff mask.
template <int LAW>
__device__ __forceinline__ float law_g(float r2, float rsm2) {
  const float y = rsqrtf(r2 + rsm2);
  return fmaf(y, y * y, neg_poly<LAW>(r2));
}

// -p'(r2), the derivative of the law's polynomial, negated.
template <int LAW>
__device__ __forceinline__ float neg_dpoly(float r2);

template <>
__device__ __forceinline__ float neg_dpoly<LAW_POLY6>(float r2) {
  float q = -6.0f * static_cast<float>(0.000000147305);
  q = fmaf(q, r2, -5.0f * static_cast<float>(-0.00000663394));
  q = fmaf(q, r2, -4.0f * static_cast<float>(0.000132336));
  q = fmaf(q, r2, -3.0f * static_cast<float>(-0.00159485));
  q = fmaf(q, r2, -2.0f * static_cast<float>(0.0133122));
  q = fmaf(q, r2, -static_cast<float>(-0.0783394));
  return q;
}

template <>
__device__ __forceinline__ float neg_dpoly<LAW_POLY5_STEP16>(float r2) {
  float q = -5.0f * static_cast<float>(-0.00000147177);
  q = fmaf(q, r2, -4.0f * static_cast<float>(0.0000605491));
  q = fmaf(q, r2, -3.0f * static_cast<float>(-0.00109313));
  q = fmaf(q, r2, -2.0f * static_cast<float>(0.0114808));
  q = fmaf(q, r2, -static_cast<float>(-0.0750978));
  return q;
}

// Whether a pair at squared distance r2 contributes (the reference's
// updateq and the law's own range, folded into one strict threshold rcut2;
// Step16_int also drops r2 == 0).
template <int LAW>
__device__ __forceinline__ bool in_range(float r2, float rcut2) {
  if (LAW == LAW_POLY5_STEP16) return r2 < rcut2 && r2 > 0.0f;
  return r2 < rcut2;
}

// 1/sqrt(s), approximate, subnormals flushed: s >= rsm^2 is a normal number
// for every law with softening, and the flush saves the subnormal rescaling.
__device__ __forceinline__ float rsqrt_ftz(float s) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(s));
  return y;
}

// One pair in the s form (batched kernel): FMA chain from rsm^2 straight to
// s, polynomial in s, weight zeroed outside the cutoff (and, for Step16, at
// r2 == 0).
template <bool DROP_SELF>
__device__ __forceinline__ void pair_acc_s(float xi, float yi, float zi, const float4 pj,
                                           const LawS &L, float &ax, float &ay, float &az) {
  const float dx = pj.x - xi;
  const float dy = pj.y - yi;
  const float dz = pj.z - zi;
  const float s = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, L.rsm2)));
  const float y = rsqrt_ftz(s);
  float q = L.nb[6];
  q = fmaf(q, s, L.nb[5]);
  q = fmaf(q, s, L.nb[4]);
  q = fmaf(q, s, L.nb[3]);
  q = fmaf(q, s, L.nb[2]);
  q = fmaf(q, s, L.nb[1]);
  q = fmaf(q, s, L.nb[0]);
  float w = pj.w * fmaf(y, y * y, q);
  const bool in = DROP_SELF ? (s < L.scut && s > L.rsm2) : (s < L.scut);
  w = in ? w : 0.f;
  ax = fmaf(w, dx, ax);
  ay = fmaf(w, dy, ay);
  az = fmaf(w, dz, az);
}

// Two pairs at once in the s form, on the packed FP32 pipe operations of
// sm_100+ (__ffma2_rn and friends: each component rounds as the scalar
// operation does): particle i against list entries a and b, given as
// A = (x_a, x_b, y_a, y_b) and B = (z_a, z_b, m_a, m_b).  (nxi, nyi, nzi) hold
// -x_i twice; x_j + (-x_i) is x_j - x_i exactly.  The accumulators keep the a
// and b sums apart.
template <bool DROP_SELF>
__device__ __forceinline__ void pair2_acc_s(float2 nxi, float2 nyi, float2 nzi, const float4 A,
                                            const float4 B, const LawS &L, float2 &ax,
                                            float2 &ay, float2 &az) {
  const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nxi);
  const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nyi);
  const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nzi);
  float2 s = __ffma2_rn(dz, dz, make_float2(L.rsm2, L.rsm2));
  s = __ffma2_rn(dy, dy, s);
  s = __ffma2_rn(dx, dx, s);
  const float2 y = make_float2(rsqrt_ftz(s.x), rsqrt_ftz(s.y));
  float2 q = make_float2(L.nb[6], L.nb[6]);
  q = __ffma2_rn(q, s, make_float2(L.nb[5], L.nb[5]));
  q = __ffma2_rn(q, s, make_float2(L.nb[4], L.nb[4]));
  q = __ffma2_rn(q, s, make_float2(L.nb[3], L.nb[3]));
  q = __ffma2_rn(q, s, make_float2(L.nb[2], L.nb[2]));
  q = __ffma2_rn(q, s, make_float2(L.nb[1], L.nb[1]));
  q = __ffma2_rn(q, s, make_float2(L.nb[0], L.nb[0]));
  float2 w = __fmul2_rn(make_float2(B.z, B.w), __ffma2_rn(y, __fmul2_rn(y, y), q));
  const bool ina = DROP_SELF ? (s.x < L.scut && s.x > L.rsm2) : (s.x < L.scut);
  const bool inb = DROP_SELF ? (s.y < L.scut && s.y > L.rsm2) : (s.y < L.scut);
  w.x = ina ? w.x : 0.f;
  w.y = inb ? w.y : 0.f;
  ax = __ffma2_rn(w, dx, ax);
  ay = __ffma2_rn(w, dy, ay);
  az = __ffma2_rn(w, dz, az);
}

// -p(r2) and -p'(r2) of the law on two values at once (packed FP32), the
// same coefficients and Horner order as neg_poly / neg_dpoly.
template <int LAW>
__device__ __forceinline__ float2 neg_poly2(float2 r2);
template <>
__device__ __forceinline__ float2 neg_poly2<LAW_POLY6>(float2 r2) {
  const float c[7] = {-static_cast<float>(0.000000147305), -static_cast<float>(-0.00000663394),
                      -static_cast<float>(0.000132336),    -static_cast<float>(-0.00159485),
                      -static_cast<float>(0.0133122),      -static_cast<float>(-0.0783394),
                      -static_cast<float>(0.271431)};
  float2 q = make_float2(c[0], c[0]);
#pragma unroll
  for (int k = 1; k < 7; ++k) q = __ffma2_rn(q, r2, make_float2(c[k], c[k]));
  return q;
}
template <>
__device__ __forceinline__ float2 neg_poly2<LAW_POLY5_STEP16>(float2 r2) {
  const float c[6] = {-static_cast<float>(-0.00000147177), -static_cast<float>(0.0000605491),
                      -static_cast<float>(-0.00109313),    -static_cast<float>(0.0114808),
                      -static_cast<float>(-0.0750978),     -static_cast<float>(0.269327)};
  float2 q = make_float2(c[0], c[0]);
#pragma unroll
  for (int k = 1; k < 6; ++k) q = __ffma2_rn(q, r2, make_float2(c[k], c[k]));
  return q;
}
// -2 p'(r2) of the law on two values at once (packed FP32): neg_dpoly's
// coefficients doubled (exactly) and its Horner order, so the result is
// exactly twice neg_dpoly's.
template <int LAW>
__device__ __forceinline__ float2 neg_dpoly2_x2(float2 r2);
template <>
__device__ __forceinline__ float2 neg_dpoly2_x2<LAW_POLY6>(float2 r2) {
  const float c[6] = {-12.0f * static_cast<float>(0.000000147305),
                      -10.0f * static_cast<float>(-0.00000663394),
                      -8.0f * static_cast<float>(0.000132336),
                      -6.0f * static_cast<float>(-0.00159485),
                      -4.0f * static_cast<float>(0.0133122), -2.0f * static_cast<float>(-0.0783394)};
  float2 q = make_float2(c[0], c[0]);
#pragma unroll
  for (int k = 1; k < 6; ++k) q = __ffma2_rn(q, r2, make_float2(c[k], c[k]));
  return q;
}
template <>
__device__ __forceinline__ float2 neg_dpoly2_x2<LAW_POLY5_STEP16>(float2 r2) {
  const float c[5] = {-10.0f * static_cast<float>(-0.00000147177),
                      -8.0f * static_cast<float>(0.0000605491),
                      -6.0f * static_cast<float>(-0.00109313),
                      -4.0f * static_cast<float>(0.0114808), -2.0f * static_cast<float>(-0.0750978)};
  float2 q = make_float2(c[0], c[0]);
#pragma unroll
  for (int k = 1; k < 5; ++k) q = __ffma2_rn(q, r2, make_float2(c[k], c[k]));
  return q;
}

// The adjoint pair term for two pairs at once: with e = x_j - x_i,
// M = w (g I + 2 g' e e^T), w = w_i m_j, returns M u (u: particle i's
// cotangent), zero where `on` is false.  Packed FP32 as pair2_acc_s.
// With MB, *mb also receives the mass cotangent of the two entries,
// d (u . dv_i) / d m_j = w_i g (d . u) (wi: fcoeff m_i, or fcoeff for Step16).
template <int LAW, bool MB = false>
__device__ __forceinline__ void vjp2_term(float2 ex, float2 ey, float2 ez, float2 w, float2 u0,
                                          float2 u1, float2 u2, float rsm2, bool on_a, bool on_b,
                                          float2 &vx, float2 &vy, float2 &vz,
                                          float2 wi = make_float2(0.f, 0.f),
                                          float2 *mb = nullptr) {
  const float2 r2 = __ffma2_rn(ex, ex, __ffma2_rn(ey, ey, __fmul2_rn(ez, ez)));
  const float2 s = __fadd2_rn(r2, make_float2(rsm2, rsm2));
  const float2 y = make_float2(rsqrt_ftz(s.x), rsqrt_ftz(s.y));
  const float2 y2 = __fmul2_rn(y, y);
  const float2 g = __ffma2_rn(y, y2, neg_poly2<LAW>(r2));
  // 2 g': the factors 2 folded into the constants (exact)
  const float2 gp2 = __ffma2_rn(__fmul2_rn(make_float2(-3.f, -3.f), y2), __fmul2_rn(y2, y),
                                neg_dpoly2_x2<LAW>(r2));
  const float2 du = __ffma2_rn(ex, u0, __ffma2_rn(ey, u1, __fmul2_rn(ez, u2)));
  float2 a = __fmul2_rn(w, g);
  float2 bq = __fmul2_rn(w, __fmul2_rn(gp2, du));
  a.x = on_a ? a.x : 0.f;
  a.y = on_b ? a.y : 0.f;
  bq.x = on_a ? bq.x : 0.f;
  bq.y = on_b ? bq.y : 0.f;
  vx = __ffma2_rn(a, u0, __fmul2_rn(bq, ex));
  vy = __ffma2_rn(a, u1, __fmul2_rn(bq, ey));
  vz = __ffma2_rn(a, u2, __fmul2_rn(bq, ez));
  if (MB) {
    float2 t = __fmul2_rn(__fmul2_rn(wi, g), du);
    t.x = on_a ? t.x : 0.f;
    t.y = on_b ? t.y : 0.f;
    *mb = t;
  }
}

// One pair: accumulates m_j g(r2) d into (ax, ay, az).
template <int LAW>
__device__ __forceinline__ void pair_acc(float xi, float yi, float zi, const float4 pj, float rsm2,
                                         float rcut2, float &ax, float &ay, float &az) {
  const float dx = pj.x - xi;
  const float dy = pj.y - yi;
  const float dz = pj.z - zi;
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float g = law_g<LAW>(r2, rsm2);
  const float w = in_range<LAW>(r2, rcut2) ? pj.w * g : 0.0f;
  ax = fmaf(w, dx, ax);
  ay = fmaf(w, dy, ay);
  az = fmaf(w, dz, az);
}

#endif  // __CUDACC__

// Launchers (sr_kernels.cu).  All take the stream to launch on and return
// the launch status.
// Counts the (leaf particle, list entry) pairs with r2 < rcut2 over the
// index lists (r2 rounded as the reference computes it, no fused
// multiply-add), added into *count.
cudaError_t launch_count_in_cutoff(const float4 *pos, const LeafDesc *leaves, int64_t nleaves,
                                   const int32_t *idx, float rcut2, unsigned long long *count,
                                   cudaStream_t s);

cudaError_t launch_expand_segments(const SegDesc *segs, int64_t nsegs, int32_t *idx,
                                   cudaStream_t s);
// threads: CTA size, i.e. threads per leaf (32, 64 or 128).
cudaError_t launch_leaf_plain(int law, int threads, const float4 *pos, const LeafDesc *leaves,
                              int64_t nleaves, const int32_t *idx, float *vx, float *vy, float *vz,
                              float fcoeff, float rsm2, float rcut2, cudaStream_t s);
cudaError_t launch_ffma_probe(float *out, int blocks, int threads, int iters, cudaStream_t s);
// Persistent batched kernel: `ctas` CTAs (0 = size from occupancy) pull
// items through the counter queue[0] (zero at launch); queue[1] receives the
// number of (particle, entry) pairs actually evaluated after the box test.
// group: particles per group of the items (16 or 32).
cudaError_t launch_pairs_batched(int law, int group, const float4 *pos, const PairItem *items,
                                 int64_t nitems, const int32_t *gidx, const int32_t *idx,
                                 float *vx, float *vy, float *vz, float fcoeff, float rsm2,
                                 float rcut2, float rcull2, unsigned long long *queue, int ctas,
                                 cudaStream_t s);
// The batched kernel over the items of several boxes (items of box b carry
// b << 8 in flags), one persistent launch; queue as above.
cudaError_t launch_pairs_batched_multi(int law, int group, const BoxDesc *boxes,
                                       const PairItem *items, int64_t nitems,
                                       unsigned long long *queue, int ctas, cudaStream_t s);
// Copies n items, tagging them with box b.
cudaError_t launch_tag_items(const PairItem *in, PairItem *out, int64_t n, int box,
                             cudaStream_t s);
// CTAs of the batched kernel that fit on the device at once.
int batched_resident_ctas(int device);

// Vector-Jacobian product of the kick dv_i = fcoeff m_i sum_j m_j g(r2) d_ij
// with respect to positions, over the same work items: for cotangent u (tree
// order, 3 x n), adds (d dv / d x)^T u into xbar (3 arrays of ntab entries:
// particles, then pseudo-particle slots).  Self entries are skipped.  With mb
// (ntab floats), also adds d (u . dv) / d m_j for every table entry j >= npart
// (the 12-point pseudo-particles' masses).
cudaError_t launch_pairs_vjp(int law, const float4 *pos, const PairItem *items, int64_t nitems,
                             const int32_t *gidx, const int32_t *idx, const float *ux,
                             const float *uy, const float *uz, float *xbx, float *xby, float *xbz,
                             float fcoeff, float rsm2, float rcut2, float rcull2,
                             unsigned long long *queue, int ctas, cudaStream_t s,
                             float *mb = nullptr, int64_t npart = 0);
// launch_pairs_vjp over the items of several boxes (items of box b carry
// b << 8 in flags), one persistent launch; queue as above.
cudaError_t launch_pairs_vjp_multi(int law, const VjpBoxDesc *boxes, const PairItem *items,
                                   int64_t nitems, unsigned long long *queue, int ctas,
                                   cudaStream_t s, bool mass_cotangents = false);
cudaError_t launch_force_law(int law, const float *r2, float *g, int64_t n, float rsm2, float rcut2,
                             cudaStream_t s);

}  // namespace hsr
