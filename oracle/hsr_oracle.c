/*
 * hsr_oracle.c -- CPU restatement of HACC's RCBForceTree short-range hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle of the GPU library and the CPU baseline
 * it is timed beside.  Never linked into or called by the product library.
 *
 * Floating point: every expression keeps the reference's operation order and
 * operand types (float vs double), and the file is compiled with
 * -ffp-contract=off so no multiply-add is fused, exactly as the reference
 * behaves on x86-64.  With the same libm, results are bit-identical to the
 * reference build in oracle/_ref (tests/test_oracle_pin.py checks this).
 *
 * Parallel structure follows the reference so the CPU baseline is timed on the
 * same shape of work: two-thread nested sections per split during the build,
 * one OpenMP task per processed leaf, and a nested parallel loop over the leaf
 * particles inside the pair kernel.
 */
#include "hsr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Force laws (src/halo_finder/ForceLaw.cxx)                                 */
/* ------------------------------------------------------------------------- */

/* FGrid::m_rmax (ForceLaw.cxx:32), stored as float. */
#define ORA_RMAX 3.116326355f

/* FGridEvalPoly coefficients, POLY_ORDER 6 (ForceLaw.cxx:98-104), as the
 * float array m_a[7] holds them. */
static const float k_poly6[7] = {0.271431f,     -0.0783394f,    0.0133122f,
                                 -0.00159485f,  0.000132336f,   -0.00000663394f,
                                 0.000000147305f};
/* Step16_int coefficients (BGQStep16.c:40-45, 167), used in double there. */
static const double k_poly5[6] = {0.269327, -0.0750978, 0.0114808,
                                  -0.00109313, 0.0000605491, -0.00000147177};

typedef struct ora_law {
  int kind;
  float rsm2;   /* ForceLawSR::m_rsm2 = rsm*rsm (ForceLaw.cxx:177)          */
  float r2min;  /* FGridEvalPoly::r2min() = 0                              */
  float r2max;  /* rmax()*rmax() (ForceLaw.cxx:130, ForceLaw.h:59)         */
  double rsm2d; /* Step16: mp_rsm2 is passed as float, used as double      */
} ora_law;

static void law_init(ora_law *L, int kind, float rsm) {
  L->kind = kind;
  L->rsm2 = rsm * rsm;
  L->r2min = 0.0f;
  L->r2max = ORA_RMAX * ORA_RMAX;
  L->rsm2d = (double)(rsm * rsm);
}

/* FGridEvalPoly::eval (ForceLaw.cxx:137-141). */
static float poly6_eval(const ora_law *L, float r2) {
  const float *a = k_poly6;
  float ret = a[0] + r2 * (a[1] + r2 * (a[2] + r2 * (a[3] + r2 * (a[4] + r2 * (a[5] + r2 * a[6])))));
  return ret * (r2 >= L->r2min) * (r2 <= L->r2max);
}

/* ForceLawSR::f_over_r (ForceLaw.cxx:187-192).  Called through a function
 * pointer from the pair loop, as the reference calls it through a virtual. */
static float sr_f_over_r(const ora_law *L, float r2) {
  float ret = powf(r2 + L->rsm2, -1.5f) - poly6_eval(L, r2);
  ret *= (r2 >= L->r2min) * (r2 <= L->r2max);
  return ret;
}

typedef float (*ora_law_fn)(const ora_law *, float);

float ora_law_f32(int law, float rsm, float r2) {
  ora_law L;
  law_init(&L, law, rsm);
  if (law == ORA_LAW_POLY5_STEP16) {
    double d = r2;
    double p = k_poly5[0] + d * (k_poly5[1] + d * (k_poly5[2] + d * (k_poly5[3] + d * (k_poly5[4] + d * k_poly5[5]))));
    return (float)(pow(d + L.rsm2d, -1.5) - p);
  }
  return sr_f_over_r(&L, r2);
}

double ora_law_f64(int law, double rsm, double r2) {
  double rs2 = rsm * rsm;
  double p;
  if (law == ORA_LAW_POLY5_STEP16) {
    p = k_poly5[0] + r2 * (k_poly5[1] + r2 * (k_poly5[2] + r2 * (k_poly5[3] + r2 * (k_poly5[4] + r2 * k_poly5[5]))));
  } else {
    const float *a = k_poly6;
    p = (double)a[0] + r2 * ((double)a[1] + r2 * ((double)a[2] + r2 * ((double)a[3] + r2 * ((double)a[4] + r2 * ((double)a[5] + r2 * (double)a[6])))));
  }
  double s = r2 + rs2;
  return 1.0 / (s * sqrt(s)) - p;  /* s^-1.5 */
}

double ora_law_dg_f64(int law, double rsm, double r2) {
  double rs2 = rsm * rsm;
  double dp = 0.0;
  if (law == ORA_LAW_POLY5_STEP16) {
    for (int k = 5; k >= 1; --k) dp = dp * r2 + k * k_poly5[k];
  } else {
    for (int k = 6; k >= 1; --k) dp = dp * r2 + k * (double)k_poly6[k];
  }
  double s = r2 + rs2;
  return -1.5 / (s * s * sqrt(s)) - dp;  /* -1.5 s^-2.5 */
}

/* ------------------------------------------------------------------------- */
/* Tree nodes (RCBForceTree.h:131-147) in a chunked pool so that concurrent  */
/* allocation never moves a node another thread is using.                    */
/* ------------------------------------------------------------------------- */

/* Children: c[0], c[1] (left, right) for the RCB tree, c[0..7] for the RCO
 * octree; 0 = none.  A node without children is a leaf. */
typedef struct onode {
  int64_t count, offset;
  int64_t c[8];
  float ppm[12];
  float tdr;
  float xmin[3], xmax[3], xc[3];
} onode;

#define CHUNK_BITS 13
#define CHUNK_SIZE ((int64_t)1 << CHUNK_BITS)

typedef struct opool {
  onode **chunks;
  int64_t nchunks; /* capacity of the chunk-pointer array */
  int64_t size;    /* nodes handed out */
#ifdef _OPENMP
  omp_lock_t lock;
#endif
} opool;

static inline onode *NODE(const opool *p, int64_t i) {
  return p->chunks[i >> CHUNK_BITS] + (i & (CHUNK_SIZE - 1));
}

static int pool_init(opool *p, int64_t max_nodes) {
  p->nchunks = (max_nodes >> CHUNK_BITS) + 2;
  p->chunks = (onode **)calloc((size_t)p->nchunks, sizeof(onode *));
  p->size = 0;
#ifdef _OPENMP
  omp_init_lock(&p->lock);
#endif
  return p->chunks != NULL;
}

static void pool_free(opool *p) {
  if (!p->chunks) return;
  for (int64_t c = 0; c < p->nchunks; ++c) free(p->chunks[c]);
  free(p->chunks);
  p->chunks = NULL;
#ifdef _OPENMP
  omp_destroy_lock(&p->lock);
#endif
}

/* Hands out k consecutive zeroed nodes; -1 when out of memory. */
static int64_t pool_alloc(opool *p, int k) {
  int64_t first;
#ifdef _OPENMP
  omp_set_lock(&p->lock);
#endif
  first = p->size;
  p->size += k;
  for (int64_t i = first; i < first + k; ++i) {
    int64_t c = i >> CHUNK_BITS;
    if (c >= p->nchunks) { first = -1; break; }
    if (!p->chunks[c]) {
      p->chunks[c] = (onode *)calloc((size_t)CHUNK_SIZE, sizeof(onode));
      if (!p->chunks[c]) { first = -1; break; }
    }
  }
#ifdef _OPENMP
  omp_unset_lock(&p->lock);
#endif
  if (first >= 0)
    for (int i = 0; i < k; ++i) memset(NODE(p, first + i), 0, sizeof(onode));
  return first;
}

/* ------------------------------------------------------------------------- */
/* Pseudo-particle geometry                                                  */
/* ------------------------------------------------------------------------- */

/* Unit points of the pseudo-particle designs (RCBForceTree.cxx:134-144 for
 * one point at the centre of mass, :227-272 for the 12 icosahedron vertices
 * of Hardin and Sloane).  The vertex order fixes the list order, so it is the
 * reference's order. */
#define ICO_A 0.525731112119134f
#define ICO_B 0.85065080835204f
static const float k_ico[12][3] = {
    {0, ICO_B, ICO_A},   {0, ICO_B, -ICO_A},  {ICO_A, 0, ICO_B},   {-ICO_A, 0, ICO_B},
    {ICO_B, ICO_A, 0},   {-ICO_B, ICO_A, 0},  {0, -ICO_B, -ICO_A}, {0, -ICO_B, ICO_A},
    {-ICO_A, 0, -ICO_B}, {ICO_A, 0, -ICO_B},  {-ICO_B, -ICO_A, 0}, {ICO_B, -ICO_A, 0}};
static const float k_mono[1][3] = {{0, 0, 0}};

static const float (*design(int tdpts))[3] { return tdpts == 12 ? k_ico : k_mono; }

/* std::min as the reference uses it: (b < a) ? b : a. */
static inline float smin(float a, float b) { return (b < a) ? b : a; }

/* pptdr (RCBForceTree.cxx:519-523): distance from the centre of mass to the
 * nearest bounding-box face. */
static float pptdr(const float *xmin, const float *xmax, const float *xc) {
  return smin(xmax[0] - xc[0],
              smin(xmax[1] - xc[1],
                   smin(xmax[2] - xc[2],
                        smin(xc[0] - xmin[0], smin(xc[1] - xmin[1], xc[2] - xmin[2])))));
}

/* pppts (RCBForceTree.cxx:525-534). */
static void pppts(int tdpts, float tdr, const float *xc, float *ppx, float *ppy, float *ppz) {
  const float (*d)[3] = design(tdpts);
  for (int i = 0; i < tdpts; ++i) {
    ppx[i] = tdr * d[i][0] + xc[0];
    ppy[i] = tdr * d[i][1] + xc[1];
    ppz[i] = tdr * d[i][2] + xc[2];
  }
}

/* pp (RCBForceTree.cxx:536-569): adds the pseudo-particle masses that
 * reproduce the monopole, dipole and quadrupole moments of `count` sources. */
static void pp_accum(int tdpts, int64_t count, const float *xx, const float *yy,
                     const float *zz, const float *mass, const float *xc,
                     const float *ppx, const float *ppy, const float *ppz,
                     float *ppm, float tdr) {
  float K = (float)tdpts;
  float odr0 = 1 / K;
  for (int i = 0; i < count; ++i) {
    float xi = xx[i] - xc[0];
    float yi = yy[i] - xc[1];
    float zi = zz[i] - xc[2];
    float ri = sqrtf(xi * xi + yi * yi + zi * zi);
    for (int j = 0; j < tdpts; ++j) {
      float xj = ppx[j] - xc[0];
      float yj = ppy[j] - xc[1];
      float zj = ppz[j] - xc[2];
      float rj2 = xj * xj + yj * yj + zj * zj;
      float odr1 = 0, odr2 = 0;
      if (rj2 != 0) {
        float rj = sqrtf(rj2);
        float aij = (xi * xj + yi * yj + zi * zj) / (ri * rj);
        odr1 = (3 / K) * (ri / tdr) * aij;
        odr2 = (float)((double)((5 / K) * (ri / tdr) * (ri / tdr)) * 0.5 * (double)(3 * aij * aij - 1));
      }
      ppm[j] += mass[i] * (odr0 + odr1 + odr2);
    }
  }
}

/* cm, generic path (src/halo_finder/BGQCM.c:181-212): tight bounding box and
 * the mass-weighted centre, accumulated in double in array order. */
static void cm(int count, const float *xx, const float *yy, const float *zz,
               const float *mass, float *xmin, float *xmax, float *xc) {
  double x = 0, y = 0, z = 0, m = 0;
  for (int i = 0; i < count; ++i) {
    if (i == 0) {
      xmin[0] = xmax[0] = xx[0];
      xmin[1] = xmax[1] = yy[0];
      xmin[2] = xmax[2] = zz[0];
    } else {
      xmin[0] = fminf(xmin[0], xx[i]);
      xmax[0] = fmaxf(xmax[0], xx[i]);
      xmin[1] = fminf(xmin[1], yy[i]);
      xmax[1] = fmaxf(xmax[1], yy[i]);
      xmin[2] = fminf(xmin[2], zz[i]);
      xmax[2] = fmaxf(xmax[2], zz[i]);
    }
    float w = mass[i];
    x += w * xx[i];
    y += w * yy[i];
    z += w * zz[i];
    m += w;
  }
  xc[0] = (float)(x / m);
  xc[1] = (float)(y / m);
  xc[2] = (float)(z / m);
}

/* ------------------------------------------------------------------------- */
/* Build (RCBForceTree.cxx:623-918)                                          */
/* ------------------------------------------------------------------------- */

typedef struct obuild {
  opool pool;
  float *x, *y, *z, *vx, *vy, *vz, *m, *phi;
  int64_t *id;
  uint16_t *mask;
  int tdpts;
  int64_t nd;
  float ppc;
  int failed;
} obuild;

/* partition (RCBForceTree.cxx:623-672): collects the indices with key < pv in
 * order, then swaps the j-th of them into slot j, all ten arrays alike.  The
 * result keeps the "left" particles in their original order; the others end
 * wherever the swap chain leaves them. */
static int64_t partition_swap(int64_t n, float *key, float *o1, float *o2, float *vx,
                              float *vy, float *vz, float *mass, float *phi,
                              int64_t *id, uint16_t *mask, float pv) {
  int32_t *idx = (int32_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
  int32_t is = 0;
  for (int32_t i = 0; i < n; ++i)
    if (key[i] < pv) idx[is++] = i;
  for (int32_t j = 0; j < is; ++j) {
    int32_t i = idx[j];
    float t;
    int64_t ti;
    uint16_t tm;
    t = mass[i]; mass[i] = mass[j]; mass[j] = t;
    t = phi[i]; phi[i] = phi[j]; phi[j] = t;
    tm = mask[i]; mask[i] = mask[j]; mask[j] = tm;
    ti = id[i]; id[i] = id[j]; id[j] = ti;
  }
  for (int32_t j = 0; j < is; ++j) {
    int32_t i = idx[j];
    float t;
    t = key[i]; key[i] = key[j]; key[j] = t;
    t = o1[i]; o1[i] = o1[j]; o1[j] = t;
    t = o2[i]; o2[i] = o2[j]; o2[j] = t;
    t = vx[i]; vx[i] = vx[j]; vx[j] = t;
    t = vy[i]; vy[i] = vy[j]; vy[j] = t;
    t = vz[i]; vz[i] = vz[j]; vz[j] = t;
  }
  free(idx);
  return is;
}

static void build_node(obuild *B, int64_t tl);

/* createRCBForceSubtree (RCBForceTree.cxx:689-775). */
static void split_node(obuild *B, int d, int64_t tl, int64_t tlcl, int64_t tlcr) {
  onode *T = NODE(&B->pool, tl);
  float *key = d == 0 ? B->x : d == 1 ? B->y : B->z;
  float *o1 = d == 0 ? B->y : d == 1 ? B->z : B->x;
  float *o2 = d == 0 ? B->z : d == 1 ? B->x : B->y;
  int64_t off = T->offset;
  float split = T->xc[d];
  int64_t is = partition_swap(T->count, key + off, o1 + off, o2 + off, B->vx + off,
                              B->vy + off, B->vz + off, B->m + off, B->phi + off,
                              B->id + off, B->mask + off, split);
  if (is == 0 || is == T->count) return;

  onode *L = NODE(&B->pool, tlcl), *R = NODE(&B->pool, tlcr);
  L->count = is;
  R->count = T->count - is;
  T->c[0] = tlcl;
  L->offset = off;
  L->xmax[d] = split;
  T->c[1] = tlcr;
  R->offset = off + is;
  R->xmin[d] = split;
#ifdef _OPENMP
#pragma omp parallel sections num_threads(2)
  {
#pragma omp section
    build_node(B, tlcl);
#pragma omp section
    build_node(B, tlcr);
  }
#else
  build_node(B, tlcl);
  build_node(B, tlcr);
#endif
}

/* Adds a child's contribution to its parent's pseudo-particle masses
 * (RCBForceTree.cxx:866-889): the child's own particles when it has no more
 * than tdpts of them, otherwise its pseudo-particles. */
static void pp_from_child(obuild *B, const onode *T, const onode *C, const float *ppx,
                          const float *ppy, const float *ppz, float *ppm) {
  int k = B->tdpts;
  if (C->count <= k) {
    int64_t o = C->offset;
    pp_accum(k, C->count, B->x + o, B->y + o, B->z + o, B->m + o, T->xc, ppx, ppy,
             ppz, ppm, T->tdr);
  } else {
    float cx[12], cy[12], cz[12];
    pppts(k, C->tdr, C->xc, cx, cy, cz);
    pp_accum(k, k, cx, cy, cz, C->ppm, T->xc, ppx, ppy, ppz, ppm, T->tdr);
  }
}

/* createRCBForceTreeInParallel (RCBForceTree.cxx:778-890). */
static void build_node(obuild *B, int64_t tl) {
  onode *T = NODE(&B->pool, tl);
  int64_t cnt = T->count, off = T->offset;
  int k = B->tdpts;

  cm((int)cnt, B->x + off, B->y + off, B->z + off, B->m + off, T->xmin, T->xmax, T->xc);

  if (cnt <= B->nd) {
    T->tdr = B->ppc * pptdr(T->xmin, T->xmax, T->xc);
    memset(T->ppm, 0, sizeof(T->ppm));
    if (cnt > k) {
      float ppx[12], ppy[12], ppz[12];
      pppts(k, T->tdr, T->xc, ppx, ppy, ppz);
      pp_accum(k, cnt, B->x + off, B->y + off, B->z + off, B->m + off, T->xc, ppx,
               ppy, ppz, T->ppm, T->tdr);
    }
    return;
  }

  int64_t tlcl = pool_alloc(&B->pool, 2);
  if (tlcl < 0) { B->failed = 1; return; }
  int64_t tlcr = tlcl + 1;
  onode *L = NODE(&B->pool, tlcl), *R = NODE(&B->pool, tlcr);
  for (int i = 0; i < 3; ++i) {
    L->xmin[i] = R->xmin[i] = T->xmin[i];
    L->xmax[i] = R->xmax[i] = T->xmax[i];
  }

  /* Longest edge; ties go to the later axis (RCBForceTree.cxx:837-852). */
  float xlen[3];
  for (int i = 0; i < 3; ++i) xlen[i] = T->xmax[i] - T->xmin[i];
  int d;
  if (xlen[0] > xlen[1] && xlen[0] > xlen[2]) d = 0;
  else if (xlen[1] > xlen[2]) d = 1;
  else d = 2;

  split_node(B, d, tl, tlcl, tlcr);

  float ppx[12], ppy[12], ppz[12];
  T->tdr = B->ppc * pptdr(T->xmin, T->xmax, T->xc);
  pppts(k, T->tdr, T->xc, ppx, ppy, ppz);
  memset(T->ppm, 0, sizeof(T->ppm));
  if (L->count > 0) pp_from_child(B, T, L, ppx, ppy, ppz, T->ppm);
  if (R->count > 0) pp_from_child(B, T, R, ppx, ppy, ppz, T->ppm);
}

/* ------------------------------------------------------------------------- */
/* RCO octree build (RCOForceTree.cxx:580-738)                               */
/* ------------------------------------------------------------------------- */

static int is_leaf(const onode *N) {
  for (int i = 0; i < 8; ++i)
    if (N->c[i] > 0) return 0;
  return 1;
}

static void swap10(obuild *B, int64_t a, int64_t b) {
  float t;
  int64_t ti;
  uint16_t tm;
#define SWAPF(arr) t = B->arr[a]; B->arr[a] = B->arr[b]; B->arr[b] = t
  SWAPF(x); SWAPF(y); SWAPF(z); SWAPF(vx); SWAPF(vy); SWAPF(vz); SWAPF(m); SWAPF(phi);
#undef SWAPF
  ti = B->id[a]; B->id[a] = B->id[b]; B->id[b] = ti;
  tm = B->mask[a]; B->mask[a] = B->mask[b]; B->mask[b] = tm;
}

/* partition (RCOForceTree.cxx:580-623): one pass in array order; a particle
 * of octant p < 7 (x, y, z at or above the split add 4, 2, 1) goes to the
 * end of octant p's run, the first particle of each later run moving up to
 * the end of the next run in turn; is[q] ends as the end of octant q's run. */
static void partition_oct(obuild *B, int64_t off, int64_t n, const float *pv, int64_t *is) {
  for (int q = 0; q < 7; ++q) is[q] = 0;
  for (int64_t i = 0; i < n; ++i) {
    int p = 0;
    if (B->x[off + i] >= pv[0]) p += 4;
    if (B->y[off + i] >= pv[1]) p += 2;
    if (B->z[off + i] >= pv[2]) p += 1;
    if (p >= 7) continue;
    swap10(B, off + is[6], off + i);
    for (int q = 6; q > p; --q) swap10(B, off + is[q - 1], off + is[q]);
    for (int q = p; q < 7; ++q) ++is[q];
  }
}

/* createRCOForceTreeInParallel / createRCOForceSubtree
 * (RCOForceTree.cxx:625-738): split all three axes at the centre of mass
 * into up to eight children, built depth first in order. */
static void build_node_oct(obuild *B, int64_t tl) {
  onode *T = NODE(&B->pool, tl);
  int64_t cnt = T->count, off = T->offset;
  int k = B->tdpts;

  cm((int)cnt, B->x + off, B->y + off, B->z + off, B->m + off, T->xmin, T->xmax, T->xc);

  if (cnt <= B->nd) {
    T->tdr = B->ppc * pptdr(T->xmin, T->xmax, T->xc);
    memset(T->ppm, 0, sizeof(T->ppm));
    if (cnt > k) {
      float ppx[12], ppy[12], ppz[12];
      pppts(k, T->tdr, T->xc, ppx, ppy, ppz);
      pp_accum(k, cnt, B->x + off, B->y + off, B->z + off, B->m + off, T->xc, ppx,
               ppy, ppz, T->ppm, T->tdr);
    }
    return;
  }

  int64_t c0 = pool_alloc(&B->pool, 8);
  if (c0 < 0) { B->failed = 1; return; }
  T = NODE(&B->pool, tl);
  for (int j = 0; j < 8; ++j) {
    onode *C = NODE(&B->pool, c0 + j);
    for (int i = 0; i < 3; ++i) {
      C->xmin[i] = T->xmin[i];
      C->xmax[i] = T->xmax[i];
    }
  }
  float split[3] = {T->xc[0], T->xc[1], T->xc[2]};
  int64_t is[7];
  partition_oct(B, off, cnt, split, is);
  int div = 0;
  for (int q = 0; q < 7; ++q)
    if (!(is[q] == 0 || is[q] == cnt)) div = 1;
  if (div) {
    int64_t counts[8];
    counts[0] = is[0];
    for (int q = 1; q < 7; ++q) counts[q] = is[q] - is[q - 1];
    counts[7] = cnt - is[6];
    int64_t coff = off;
    for (int j = 0; j < 8; ++j) {
      onode *C = NODE(&B->pool, c0 + j);
      C->count = counts[j];
      if (counts[j] > 0) {
        T->c[j] = c0 + j;
        C->offset = coff;
        coff += counts[j];
        build_node_oct(B, c0 + j);
        if (B->failed) return;
      }
    }
  }

  float ppx[12], ppy[12], ppz[12];
  T->tdr = B->ppc * pptdr(T->xmin, T->xmax, T->xc);
  pppts(k, T->tdr, T->xc, ppx, ppy, ppz);
  memset(T->ppm, 0, sizeof(T->ppm));
  for (int j = 0; j < 8; ++j) {
    const onode *C = NODE(&B->pool, c0 + j);
    if (C->count > 0 && T->c[j] > 0) pp_from_child(B, T, C, ppx, ppy, ppz, T->ppm);
  }
}

/* ------------------------------------------------------------------------- */
/* Walk + pair kernel (RCBForceTree.cxx:575-620, 923-1197)                   */
/* ------------------------------------------------------------------------- */

typedef struct olist {
  float *x, *y, *z, *m;
  int64_t size, cap;
} olist;

static int list_reserve(olist *L, int64_t need) {
  if (need <= L->cap) return 1;
  int64_t c = L->cap ? L->cap : 1024;
  while (c < need) c *= 2;
  float *nx = (float *)realloc(L->x, (size_t)c * sizeof(float));
  if (nx) L->x = nx;
  float *ny = (float *)realloc(L->y, (size_t)c * sizeof(float));
  if (ny) L->y = ny;
  float *nz = (float *)realloc(L->z, (size_t)c * sizeof(float));
  if (nz) L->z = nz;
  float *nm = (float *)realloc(L->m, (size_t)c * sizeof(float));
  if (nm) L->m = nm;
  if (!nx || !ny || !nz || !nm) return 0;
  L->cap = c;
  return 1;
}

static void list_free(olist *L) {
  free(L->x); free(L->y); free(L->z); free(L->m);
  memset(L, 0, sizeof(*L));
}

struct ora_result {
  ora_stats st;
  opool pool;
  int tdpts;
  ora_law law;
  float fsrrmax;
  /* processed leaves in DFS order */
  int64_t nleaves;
  int64_t *leaf_node;
  olist *lists; /* kept when keep_lists */
  const float *x, *y, *z, *m; /* borrowed, post-permutation */
  int err;
};

typedef struct owalk {
  const opool *pool;
  const float *x, *y, *z, *m;
  float *vx, *vy, *vz;
  int tdpts;
  float fsrrmax, tan_oa;
  const ora_law *law;
  ora_law_fn fl;
  float fcoeff;
  int64_t vmax;
  int do_kick;
} owalk;

/* nbody1, generic path (RCBForceTree.cxx:599-619). */
static void nbody1(int64_t count, int64_t count1, const float *xx, const float *yy,
                   const float *zz, const float *mass, const float *xx1,
                   const float *yy1, const float *zz1, const float *mass1, float *vx,
                   float *vy, float *vz, ora_law_fn fl, const ora_law *law, float fcoeff,
                   float fsrrmax) {
  float fsrrmax2 = fsrrmax * fsrrmax;
#ifdef _OPENMP
#pragma omp parallel for
#endif
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < count1; ++j) {
      float dx = xx1[j] - xx[i];
      float dy = yy1[j] - yy[i];
      float dz = zz1[j] - zz[i];
      float dist2 = dx * dx + dy * dy + dz * dz;
      float f_over_r = mass[i] * mass1[j] * fl(law, dist2);
      float updateq = 1.0f;
      updateq *= (dist2 < fsrrmax2);
      vx[i] += updateq * fcoeff * f_over_r * dx;
      vy[i] += updateq * fcoeff * f_over_r * dy;
      vz[i] += updateq * fcoeff * f_over_r * dz;
    }
}

/* Step16_int semantics (BGQStep16.c:23-189) for one leaf: per target, double
 * accumulation, 5th-order polynomial, no m_i, r2 == 0 and r2 >= fsrrmax2
 * dropped; vx += ax * fcoeff. */
static void nbody_step16(int64_t count, int64_t count1, const float *xx, const float *yy,
                         const float *zz, const float *xx1, const float *yy1,
                         const float *zz1, const float *mass1, float *vx, float *vy,
                         float *vz, double rsm2, float fcoeff, float fsrrmax) {
  double fsrrmax2 = (double)(fsrrmax * fsrrmax);
  for (int64_t i = 0; i < count; ++i) {
    double ax = 0, ay = 0, az = 0;
    for (int64_t j = 0; j < count1; ++j) {
      double dx = (double)xx1[j] - (double)xx[i];
      double dy = (double)yy1[j] - (double)yy[i];
      double dz = (double)zz1[j] - (double)zz[i];
      double r2 = dx * dx + dy * dy + dz * dz;
      if (!(r2 < fsrrmax2) || !(r2 > 0.0)) continue;
      double p = k_poly5[0] + r2 * (k_poly5[1] + r2 * (k_poly5[2] + r2 * (k_poly5[3] + r2 * (k_poly5[4] + r2 * k_poly5[5]))));
      double f = (double)mass1[j] * (pow(r2 + rsm2, -1.5) - p);
      ax += f * dx;
      ay += f * dy;
      az += f * dz;
    }
    vx[i] = vx[i] + (float)ax * fcoeff;
    vy[i] = vy[i] + (float)ay * fcoeff;
    vz[i] = vz[i] + (float)az * fcoeff;
  }
}

static int is_ancestor(const int64_t *parents, int64_t np, int64_t t) {
  /* binary_search over the root-to-leaf path (indices ascend along it) */
  int64_t lo = 0, hi = np;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (parents[mid] < t) lo = mid + 1;
    else hi = mid;
  }
  return lo < np && parents[lo] == t;
}

static int append_particles(olist *L, const owalk *W, int64_t off, int64_t cnt) {
  if (!list_reserve(L, L->size + cnt)) return 0;
  for (int64_t i = 0; i < cnt; ++i) {
    L->x[L->size + i] = W->x[off + i];
    L->y[L->size + i] = W->y[off + i];
    L->z[L->size + i] = W->z[off + i];
    L->m[L->size + i] = W->m[off + i];
  }
  L->size += cnt;
  return 1;
}

/* Closeness of a child's box to the target leaf's box along every axis
 * (RCBForceTree.cxx:1088-1123). */
static int box_close(const onode *tl, const onode *c, float fsrrmax) {
  for (int i = 0; i < 3; ++i) {
    float dist = 0;
    if (tl->xmax[i] < c->xmin[i]) dist = c->xmin[i] - tl->xmax[i];
    else if (tl->xmin[i] > c->xmax[i]) dist = tl->xmin[i] - c->xmax[i];
    if (dist > fsrrmax) return 0;
  }
  return 1;
}

/* calcInternodeForce (RCBForceTree.cxx:923-1144): builds leaf tl's list in
 * the reference's order (stack walk, self last) into L and applies nbody1.
 * Returns ORA_OK or an error code. */
static int leaf_walk(const owalk *W, int64_t tl, const int64_t *parents, int64_t np,
                     olist *L, int64_t **qbuf, int64_t *qcap) {
  const opool *P = W->pool;
  const onode *T = NODE(P, tl);
  float fsrrmax2 = W->fsrrmax * W->fsrrmax;
  int64_t qn = 0;
  int k = W->tdpts;
#define QPUSH(v)                                                              \
  do {                                                                        \
    if (qn == *qcap) {                                                        \
      *qcap = *qcap ? 2 * *qcap : 256;                                        \
      *qbuf = (int64_t *)realloc(*qbuf, (size_t)*qcap * sizeof(int64_t));     \
      if (!*qbuf) return ORA_ERR_NOMEM;                                       \
    }                                                                         \
    (*qbuf)[qn++] = (v);                                                      \
  } while (0)

  L->size = 0;
  QPUSH(0);
  while (qn > 0) {
    int64_t tln = (*qbuf)[--qn];
    const onode *N = NODE(P, tln);

    if (tln < tl && is_ancestor(parents, np, tln)) {
      for (int j = 0; j < 8; ++j) {
        int64_t c = N->c[j];
        if (c != tl && c > 0 && NODE(P, c)->count > 0) QPUSH(c);
      }
      continue;
    }

    float dx = N->xc[0] - T->xc[0];
    float dy = N->xc[1] - T->xc[1];
    float dz = N->xc[2] - T->xc[2];
    float dist2 = dx * dx + dy * dy + dz * dz;
    float sx = N->xmax[0] - N->xmin[0];
    float sy = N->xmax[1] - N->xmin[1];
    float sz = N->xmax[2] - N->xmin[2];
    float l2 = smin(sx * sx, smin(sy * sy, sz * sz));
    float dtt2 = dist2 * W->tan_oa * W->tan_oa;
    int big;
    if (l2 > dtt2) {
      big = 1;
    } else {
      /* four corner-to-opposite-corner diagonals, tan approximation
       * (RCBForceTree.cxx:988-1020) */
      big = 0;
      for (int i = 0; i < 2 && !big; ++i)
        for (int j = 0; j < 2; ++j) {
          float x1 = (i == 0 ? N->xmin : N->xmax)[0] - T->xc[0];
          float y1 = (j == 0 ? N->xmin : N->xmax)[1] - T->xc[1];
          float z1 = N->xmin[2] - T->xc[2];
          float x2 = (i == 0 ? N->xmax : N->xmin)[0] - T->xc[0];
          float y2 = (j == 0 ? N->xmax : N->xmin)[1] - T->xc[1];
          float z2 = N->xmax[2] - T->xc[2];
          float ddx = x1 - x2, ddy = y1 - y2, ddz = z1 - z2;
          float dh2 = ddx * ddx + ddy * ddy + ddz * ddz;
          if (dh2 > dtt2) { big = 1; break; }
        }
    }

    if (!big) {
      if (dist2 > fsrrmax2) continue;
      if (N->count <= k) {
        if (!append_particles(L, W, N->offset, N->count)) return ORA_ERR_NOMEM;
      } else {
        if (!list_reserve(L, L->size + k)) return ORA_ERR_NOMEM;
        pppts(k, N->tdr, N->xc, L->x + L->size, L->y + L->size, L->z + L->size);
        for (int i = 0; i < k; ++i) L->m[L->size + i] = N->ppm[i];
        L->size += k;
      }
      if (W->vmax > 0 && L->size >= W->vmax) return ORA_ERR_VMAX;
      continue;
    } else if (is_leaf(N)) {
      if (!append_particles(L, W, N->offset, N->count)) return ORA_ERR_NOMEM;
      if (W->vmax > 0 && L->size >= W->vmax) return ORA_ERR_VMAX;
      continue;
    }

    for (int j = 0; j < 8; ++j) {
      int64_t c = N->c[j];
      if (c > 0 && NODE(P, c)->count > 0 && box_close(T, NODE(P, c), W->fsrrmax)) QPUSH(c);
    }
  }
#undef QPUSH

  if (!append_particles(L, W, T->offset, T->count)) return ORA_ERR_NOMEM;
  if (W->vmax > 0 && L->size >= W->vmax) return ORA_ERR_VMAX;

  if (W->do_kick) {
    int64_t off = T->offset;
    if (W->law->kind == ORA_LAW_POLY5_STEP16)
      nbody_step16(T->count, L->size, W->x + off, W->y + off, W->z + off, L->x, L->y,
                   L->z, L->m, W->vx + off, W->vy + off, W->vz + off, W->law->rsm2d,
                   W->fcoeff, W->fsrrmax);
    else
      nbody1(T->count, L->size, W->x + off, W->y + off, W->z + off, W->m + off, L->x,
             L->y, L->z, L->m, W->vx + off, W->vy + off, W->vz + off, W->fl, W->law,
             W->fcoeff, W->fsrrmax);
  }
  return ORA_OK;
}

static double now_s(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return (double)clock() / CLOCKS_PER_SEC;
#endif
}

ora_result *ora_rcb_run(const ora_params *p, int64_t n, float *x, float *y, float *z,
                        float *vx, float *vy, float *vz, float *mass, float *phi,
                        int64_t *id, uint16_t *mask, int keep_lists, int do_kick,
                        int *err) {
  *err = ORA_OK;
  if (!p || n < 0 || (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !mass || !phi || !id || !mask)) ||
      (p->tdpts != 1 && p->tdpts != 12) || p->nd < 1 || n >= ((int64_t)1 << 31) ||
      (p->tree != ORA_TREE_RCB && p->tree != ORA_TREE_RCO)) {
    *err = ORA_ERR_ARG;
    return NULL;
  }
  ora_result *R = (ora_result *)calloc(1, sizeof(ora_result));
  if (!R) { *err = ORA_ERR_NOMEM; return NULL; }
#ifdef _OPENMP
  int nest = omp_get_max_active_levels();
  /* The reference nests a two-thread team per split (omp_set_nested(1),
   * RCBForceTree.cxx:418-421), so a deep tree asks for ~2^depth threads at
   * once.  ORA_MAX_ACTIVE_LEVELS caps the nesting for very large inputs
   * (deeper splits then run in the calling thread); the results do not
   * depend on it. */
  int levels = 64;
  {
    const char *e = getenv("ORA_MAX_ACTIVE_LEVELS");
    if (e && atoi(e) > 0) levels = atoi(e);
  }
  omp_set_max_active_levels(levels);
  if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
  R->tdpts = p->tdpts;
  R->fsrrmax = p->fsrrmax;
  law_init(&R->law, p->law, p->rsm);
  R->x = x; R->y = y; R->z = z; R->m = mass;

  /* ---- build (createRCBForceTree, RCBForceTree.cxx:892-918) ---- */
  double t0 = now_s();
  obuild B;
  memset(&B, 0, sizeof(B));
  if (!pool_init(&B.pool, (p->tree == ORA_TREE_RCO ? 8 : 2) * n + 9)) {
    free(R);
    *err = ORA_ERR_NOMEM;
    return NULL;
  }
  B.x = x; B.y = y; B.z = z; B.vx = vx; B.vy = vy; B.vz = vz; B.m = mass; B.phi = phi;
  B.id = id; B.mask = mask; B.tdpts = p->tdpts; B.nd = p->nd; B.ppc = p->ppc;
  int64_t root = pool_alloc(&B.pool, 1);
  onode *T0 = NODE(&B.pool, root);
  T0->count = n;
  T0->offset = 0;
  for (int i = 0; i < 3; ++i) { T0->xmin[i] = p->min[i]; T0->xmax[i] = p->max[i]; }
  if (p->tree == ORA_TREE_RCO) build_node_oct(&B, root);
  else build_node(&B, root);
  double t1 = now_s();
  R->pool = B.pool;
  if (B.failed) { *err = ORA_ERR_NOMEM; ora_result_free(R); return NULL; }

  /* ---- processed leaves in the DFS order of calcInternodeForces
   *      (RCBForceTree.cxx:1150-1197), each with its ancestor path ---- */
  const opool *P = &R->pool;
  int64_t cap = 1024, nl = 0;
  int64_t *leaves = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  int64_t **paths = (int64_t **)malloc((size_t)cap * sizeof(int64_t *));
  int64_t *plen = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
  int64_t *q = (int64_t *)malloc(sizeof(int64_t) * 256), qn = 0, qc = 256;
  int64_t *par = (int64_t *)malloc(sizeof(int64_t) * 256), pn = 0, pc = 256;
  q[qn++] = 0;
  while (qn > 0) {
    int64_t tl = q[qn - 1];
    const onode *N = NODE(P, tl);
    if (is_leaf(N)) {
      --qn;
      int inside = 1;
      for (int i = 0; i < 3; ++i)
        inside &= (N->xmax[i] < p->max_force[i] && N->xmax[i] > p->min_force[i]) ||
                  (N->xmin[i] < p->max_force[i] && N->xmin[i] > p->min_force[i]);
      if (inside) {
        if (nl == cap) {
          cap *= 2;
          leaves = (int64_t *)realloc(leaves, (size_t)cap * sizeof(int64_t));
          paths = (int64_t **)realloc(paths, (size_t)cap * sizeof(int64_t *));
          plen = (int64_t *)realloc(plen, (size_t)cap * sizeof(int64_t));
        }
        leaves[nl] = tl;
        paths[nl] = (int64_t *)malloc((size_t)(pn > 0 ? pn : 1) * sizeof(int64_t));
        memcpy(paths[nl], par, (size_t)pn * sizeof(int64_t));
        plen[nl] = pn;
        ++nl;
      }
    } else if (pn > 0 && par[pn - 1] == tl) {
      --pn;
      --qn;
    } else {
      if (qn + 8 > qc) { qc *= 2; q = (int64_t *)realloc(q, (size_t)qc * sizeof(int64_t)); }
      for (int j = 0; j < 8; ++j)
        if (N->c[j] > 0) q[qn++] = N->c[j];
      if (pn == pc) { pc *= 2; par = (int64_t *)realloc(par, (size_t)pc * sizeof(int64_t)); }
      par[pn++] = tl;
    }
  }
  free(q);
  free(par);

  R->nleaves = nl;
  R->leaf_node = leaves;
  R->lists = (olist *)calloc((size_t)(nl > 0 ? nl : 1), sizeof(olist));

  owalk W;
  W.pool = P; W.x = x; W.y = y; W.z = z; W.m = mass; W.vx = vx; W.vy = vy; W.vz = vz;
  W.tdpts = p->tdpts; W.fsrrmax = p->fsrrmax; W.tan_oa = tanf(p->open_angle);
  W.law = &R->law; W.fl = sr_f_over_r; W.fcoeff = p->fcoeff;
  W.vmax = p->vmax; W.do_kick = do_kick;

  int werr = ORA_OK;
  int64_t tot_entries = 0, tot_pairs = 0;
#ifdef _OPENMP
#pragma omp parallel
#pragma omp single
#endif
  {
    for (int64_t li = 0; li < nl; ++li) {
#ifdef _OPENMP
#pragma omp task firstprivate(li) shared(werr, tot_entries, tot_pairs)
#endif
      {
        olist own;
        memset(&own, 0, sizeof(own));
        olist *L = keep_lists ? &R->lists[li] : &own;
        int64_t *qb = NULL, qcp = 0;
        int e = leaf_walk(&W, leaves[li], paths[li], plen[li], L, &qb, &qcp);
        free(qb);
        int64_t cnt = NODE(P, leaves[li])->count;
#ifdef _OPENMP
#pragma omp critical(ora_tally)
#endif
        {
          if (e != ORA_OK && werr == ORA_OK) werr = e;
          tot_entries += L->size;
          tot_pairs += cnt * L->size;
        }
        if (!keep_lists) list_free(&own);
      }
    }
#ifdef _OPENMP
#pragma omp taskwait
#endif
  }
  double t2 = now_s();
  for (int64_t li = 0; li < nl; ++li) free(paths[li]);
  free(paths);
  free(plen);

  /* statistics (printStats, RCBForceTree.cxx:461-511) */
  R->st.nodes = P->size;
  for (int64_t t = 1; t < P->size; ++t) {
    const onode *N = NODE(P, t);
    if (is_leaf(N)) {
      if (N->count > 0) {
        R->st.leaves++;
        if (N->count > R->st.max_ppn) R->st.max_ppn = N->count;
      } else {
        R->st.empty_leaves++;
      }
    }
  }
  R->st.processed_leaves = nl;
  R->st.list_entries = tot_entries;
  R->st.pairs = tot_pairs;
  R->st.t_build = t1 - t0;
  R->st.t_walk = t2 - t1;
#ifdef _OPENMP
  omp_set_max_active_levels(nest);
#endif
  if (werr != ORA_OK) {
    *err = werr;
    ora_result_free(R);
    return NULL;
  }
  return R;
}

void ora_result_stats(const ora_result *r, ora_stats *st) { *st = r->st; }
int64_t ora_result_nleaves(const ora_result *r) { return r->nleaves; }

int64_t ora_result_nentries(const ora_result *r) {
  int64_t s = 0;
  for (int64_t i = 0; i < r->nleaves; ++i) s += r->lists[i].size;
  return s;
}

void ora_result_leaves(const ora_result *r, int64_t *leaf_offset, int64_t *leaf_count,
                       int64_t *list_ptr) {
  int64_t s = 0;
  for (int64_t i = 0; i < r->nleaves; ++i) {
    const onode *N = NODE(&r->pool, r->leaf_node[i]);
    leaf_offset[i] = N->offset;
    leaf_count[i] = N->count;
    list_ptr[i] = s;
    s += r->lists[i].size;
  }
  list_ptr[r->nleaves] = s;
}

void ora_result_entries(const ora_result *r, float *ex, float *ey, float *ez, float *em) {
  int64_t s = 0;
  for (int64_t i = 0; i < r->nleaves; ++i) {
    const olist *L = &r->lists[i];
    if (L->size) {
      memcpy(ex + s, L->x, (size_t)L->size * sizeof(float));
      memcpy(ey + s, L->y, (size_t)L->size * sizeof(float));
      memcpy(ez + s, L->z, (size_t)L->size * sizeof(float));
      memcpy(em + s, L->m, (size_t)L->size * sizeof(float));
    }
    s += L->size;
  }
}

int64_t ora_result_nnodes(const ora_result *r) { return r->pool.size; }

void ora_result_nodes(const ora_result *r, int64_t *count, int64_t *offset, int64_t *cl,
                      int64_t *cr, float *tdr, float *bbox9, float *ppm) {
  for (int64_t t = 0; t < r->pool.size; ++t) {
    const onode *N = NODE(&r->pool, t);
    count[t] = N->count;
    offset[t] = N->offset;
    cl[t] = N->c[0];
    cr[t] = N->c[1];
    tdr[t] = N->tdr;
    for (int i = 0; i < 3; ++i) {
      bbox9[9 * t + i] = N->xmin[i];
      bbox9[9 * t + 3 + i] = N->xmax[i];
      bbox9[9 * t + 6 + i] = N->xc[i];
    }
    for (int i = 0; i < r->tdpts; ++i) ppm[(int64_t)r->tdpts * t + i] = N->ppm[i];
  }
}

void ora_result_acc_fp64(const ora_result *r, double *ax, double *ay, double *az) {
  double rmax2 = (double)(r->fsrrmax * r->fsrrmax);
  int law = r->law.kind;
  double rsm = sqrt((double)r->law.rsm2);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t li = 0; li < r->nleaves; ++li) {
    const onode *N = NODE(&r->pool, r->leaf_node[li]);
    const olist *L = &r->lists[li];
    for (int64_t i = N->offset; i < N->offset + N->count; ++i) {
      double sx = 0, sy = 0, sz = 0;
      for (int64_t j = 0; j < L->size; ++j) {
        double dx = (double)L->x[j] - r->x[i];
        double dy = (double)L->y[j] - r->y[i];
        double dz = (double)L->z[j] - r->z[i];
        double r2 = dx * dx + dy * dy + dz * dz;
        if (!(r2 < rmax2)) continue;
        if (law == ORA_LAW_POLY5_STEP16 && !(r2 > 0)) continue;
        double w = (double)L->m[j] * ora_law_f64(law, rsm, r2);
        if (law != ORA_LAW_POLY5_STEP16) w *= (double)r->m[i];
        sx += w * dx; sy += w * dy; sz += w * dz;
      }
      ax[i] = sx; ay[i] = sy; az[i] = sz;
    }
  }
}

void ora_result_free(ora_result *r) {
  if (!r) return;
  if (r->lists)
    for (int64_t i = 0; i < r->nleaves; ++i) list_free(&r->lists[i]);
  free(r->lists);
  free(r->leaf_node);
  pool_free(&r->pool);
  free(r);
}

/* ------------------------------------------------------------------------- */
/* FP64 direct sum and FP64 VJP                                              */
/* ------------------------------------------------------------------------- */

void ora_direct_fp64(int64_t n, const float *x, const float *y, const float *z,
                     const float *mass, int law, float rsm, float fsrrmax,
                     int64_t ntargets, const int64_t *targets, double *ax, double *ay,
                     double *az) {
  double rmax2 = (double)(fsrrmax * fsrrmax);
  double rc = (double)fsrrmax;
  /* cell list with cell edge >= cutoff */
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < n; ++i) {
    double p[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) { if (p[d] < lo[d]) lo[d] = p[d]; if (p[d] > hi[d]) hi[d] = p[d]; }
  }
  int nc[3];
  for (int d = 0; d < 3; ++d) {
    nc[d] = (int)((hi[d] - lo[d]) / rc) + 1;
    if (nc[d] < 1) nc[d] = 1;
  }
  int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
  int64_t *head = (int64_t *)malloc((size_t)(ncell + 1) * sizeof(int64_t));
  int64_t *order = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t *cell = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  memset(head, 0, (size_t)(ncell + 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    int c[3];
    double p[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; ++d) {
      c[d] = (int)((p[d] - lo[d]) / rc);
      if (c[d] >= nc[d]) c[d] = nc[d] - 1;
    }
    cell[i] = ((int64_t)c[0] * nc[1] + c[1]) * nc[2] + c[2];
    head[cell[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; ++c) head[c + 1] += head[c];
  int64_t *fill = (int64_t *)malloc((size_t)(ncell + 1) * sizeof(int64_t));
  memcpy(fill, head, (size_t)(ncell + 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) order[fill[cell[i]]++] = i;
  free(fill);
  double rsmd = (double)rsm;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int64_t t = 0; t < ntargets; ++t) {
    int64_t i = targets[t];
    double xi = x[i], yi = y[i], zi = z[i];
    int c[3];
    double p[3] = {xi, yi, zi};
    for (int d = 0; d < 3; ++d) {
      c[d] = (int)((p[d] - lo[d]) / rc);
      if (c[d] >= nc[d]) c[d] = nc[d] - 1;
    }
    double sx = 0, sy = 0, sz = 0;
    for (int a = c[0] - 1; a <= c[0] + 1; ++a)
      for (int b = c[1] - 1; b <= c[1] + 1; ++b)
        for (int e = c[2] - 1; e <= c[2] + 1; ++e) {
          if (a < 0 || b < 0 || e < 0 || a >= nc[0] || b >= nc[1] || e >= nc[2]) continue;
          int64_t cc = ((int64_t)a * nc[1] + b) * nc[2] + e;
          for (int64_t k = head[cc]; k < head[cc + 1]; ++k) {
            int64_t j = order[k];
            double dx = (double)x[j] - xi, dy = (double)y[j] - yi, dz = (double)z[j] - zi;
            double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 < rmax2)) continue;
            if (law == ORA_LAW_POLY5_STEP16 && !(r2 > 0)) continue;
            double w = (double)mass[j] * ora_law_f64(law, rsmd, r2);
            if (law != ORA_LAW_POLY5_STEP16) w *= (double)mass[i];
            sx += w * dx; sy += w * dy; sz += w * dz;
          }
        }
    ax[t] = sx; ay[t] = sy; az[t] = sz;
  }
  free(head);
  free(order);
  free(cell);
}

void ora_vjp_fp64(int64_t n, const float *x, const float *y, const float *z,
                  const float *mass, int law, float rsm, float fsrrmax, double c,
                  int64_t nleaves, const int64_t *leaf_offset, const int64_t *leaf_count,
                  const int64_t *list_ptr, const int64_t *list_idx, const double *u,
                  double *xbar) {
  /* a_i = c sum_j w_ij d_ij, d = x_j - x_i, w = m_i m_j g(r2).
   * da_i/dx_j = c m_i m_j (g I + 2 g' d d^T) =: M_ij; da_i/dx_i = -sum_j M_ij.
   * xbar_j += M_ij^T u_i = M_ij u_i (symmetric); xbar_i -= M_ij u_i. */
  double rmax2 = (double)(fsrrmax * fsrrmax);
  double rsmd = (double)rsm;
  memset(xbar, 0, (size_t)(3 * n) * sizeof(double));
  for (int64_t l = 0; l < nleaves; ++l) {
    for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i) {
      const double *ui = u + 3 * i;
      for (int64_t k = list_ptr[l]; k < list_ptr[l + 1]; ++k) {
        int64_t j = list_idx[k];
        double d[3] = {(double)x[j] - x[i], (double)y[j] - y[i], (double)z[j] - z[i]};
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (!(r2 < rmax2)) continue;
        if (law == ORA_LAW_POLY5_STEP16 && !(r2 > 0)) continue;
        double mm = (double)mass[j];
        if (law != ORA_LAW_POLY5_STEP16) mm *= (double)mass[i];
        double g = ora_law_f64(law, rsmd, r2), gp = ora_law_dg_f64(law, rsmd, r2);
        double du = d[0] * ui[0] + d[1] * ui[1] + d[2] * ui[2];
        for (int a = 0; a < 3; ++a) {
          double v = c * mm * (g * ui[a] + 2.0 * gp * d[a] * du);
          xbar[3 * j + a] += v;
          xbar[3 * i + a] -= v;
        }
      }
    }
  }
}

/* Pair term weight and its derivative pieces in FP64. */
static int pair_terms(int law, double rsm, double rmax2, double mi, double mj, const double d[3],
                      double *w_g, double *w_gp) {
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (!(r2 < rmax2)) return 0;
  if (law == ORA_LAW_POLY5_STEP16 && !(r2 > 0)) return 0;
  double mm = mj * (law == ORA_LAW_POLY5_STEP16 ? 1.0 : mi);
  *w_g = mm * ora_law_f64(law, rsm, r2);
  *w_gp = mm * ora_law_dg_f64(law, rsm, r2);
  return 1;
}

void ora_vjp_fp64_tab(int64_t n, const float *tab, int64_t ntab, const int64_t *pnode_off,
                      const int64_t *pnode_cnt, int law, float rsm, float fsrrmax, double c,
                      int64_t nleaves, const int64_t *leaf_offset, const int64_t *leaf_count,
                      const int64_t *list_ptr, const int64_t *list_idx, const double *u,
                      double *xbar) {
  double rmax2 = (double)(fsrrmax * fsrrmax);
  double *xt = (double *)calloc((size_t)(3 * ntab), sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t l = 0; l < nleaves; ++l) {
    for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i) {
      const double *ui = u + 3 * i;
      double xi[3] = {tab[4 * i], tab[4 * i + 1], tab[4 * i + 2]};
      double mi = tab[4 * i + 3];
      double acc[3] = {0, 0, 0};
      for (int64_t k = list_ptr[l]; k < list_ptr[l + 1]; ++k) {
        int64_t e = list_idx[k];
        if (e == i) continue;
        double d[3] = {tab[4 * e] - xi[0], tab[4 * e + 1] - xi[1], tab[4 * e + 2] - xi[2]};
        double wg, wgp;
        if (!pair_terms(law, rsm, rmax2, mi, tab[4 * e + 3], d, &wg, &wgp)) continue;
        double du = d[0] * ui[0] + d[1] * ui[1] + d[2] * ui[2];
        for (int a = 0; a < 3; ++a) {
          double v = c * (wg * ui[a] + 2.0 * wgp * du * d[a]);
          acc[a] -= v;
#ifdef _OPENMP
#pragma omp atomic
#endif
          xt[3 * e + a] += v;
        }
      }
      for (int a = 0; a < 3; ++a) {
#ifdef _OPENMP
#pragma omp atomic
#endif
        xt[3 * i + a] += acc[a];
      }
    }
  }
  for (int64_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) xbar[3 * k + a] = xt[3 * k + a];
  /* pseudo-particles: d xc / d x_k = m_k / M */
  for (int64_t t = n; t < ntab; ++t) {
    double g[3] = {xt[3 * t], xt[3 * t + 1], xt[3 * t + 2]};
    if (g[0] == 0 && g[1] == 0 && g[2] == 0) continue;
    double M = tab[4 * t + 3];
    if (M == 0) continue;
    for (int64_t k = pnode_off[t - n]; k < pnode_off[t - n] + pnode_cnt[t - n]; ++k)
      for (int a = 0; a < 3; ++a) xbar[3 * k + a] += (double)tab[4 * k + 3] / M * g[a];
  }
  free(xt);
}

/* FP64 positions of the table: particles (tree order) then one pseudo-particle
 * per node slot at the FP64 centre of mass of the node's particles. */
static void tab64_fill(int64_t n, const double *pos, const double *m, int64_t nslots,
                       const int64_t *pnode_off, const int64_t *pnode_cnt, double *tab) {
  for (int64_t i = 0; i < n; ++i) {
    tab[4 * i] = pos[3 * i];
    tab[4 * i + 1] = pos[3 * i + 1];
    tab[4 * i + 2] = pos[3 * i + 2];
    tab[4 * i + 3] = m[i];
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (int64_t t = 0; t < nslots; ++t) {
    double M = 0, c[3] = {0, 0, 0};
    for (int64_t k = pnode_off[t]; k < pnode_off[t] + pnode_cnt[t]; ++k) {
      M += m[k];
      for (int a = 0; a < 3; ++a) c[a] += m[k] * pos[3 * k + a];
    }
    double *o = tab + 4 * (n + t);
    for (int a = 0; a < 3; ++a) o[a] = M != 0 ? c[a] / M : 0.0;
    o[3] = M;
  }
}

void ora_kick64(int64_t n, const double *pos, const double *m, int64_t nslots,
                const int64_t *pnode_off, const int64_t *pnode_cnt, int law, double rsm,
                double fsrrmax, double c, int64_t nleaves, const int64_t *leaf_offset,
                const int64_t *leaf_count, const int64_t *list_ptr, const int64_t *list_idx,
                const double *pos_cut, double *dv) {
  double rmax2 = fsrrmax * fsrrmax;
  double *tab = (double *)malloc((size_t)(4 * (n + nslots) + 4) * sizeof(double));
  double *tcut = NULL;
  tab64_fill(n, pos, m, nslots, pnode_off, pnode_cnt, tab);
  if (pos_cut) {
    tcut = (double *)malloc((size_t)(4 * (n + nslots) + 4) * sizeof(double));
    tab64_fill(n, pos_cut, m, nslots, pnode_off, pnode_cnt, tcut);
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t l = 0; l < nleaves; ++l) {
    for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i) {
      double a[3] = {0, 0, 0};
      for (int64_t k = list_ptr[l]; k < list_ptr[l + 1]; ++k) {
        int64_t e = list_idx[k];
        if (e == i) continue;
        double d[3] = {tab[4 * e] - tab[4 * i], tab[4 * e + 1] - tab[4 * i + 1],
                       tab[4 * e + 2] - tab[4 * i + 2]};
        /* the cutoff decided at the reference positions when given */
        const double *tc = tcut ? tcut : tab;
        double dc[3] = {tc[4 * e] - tc[4 * i], tc[4 * e + 1] - tc[4 * i + 1],
                        tc[4 * e + 2] - tc[4 * i + 2]};
        double rc2 = dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2];
        if (!(rc2 < rmax2)) continue;
        if (law == ORA_LAW_POLY5_STEP16 && !(rc2 > 0)) continue;
        double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double mm = tab[4 * e + 3] * (law == ORA_LAW_POLY5_STEP16 ? 1.0 : tab[4 * i + 3]);
        double wg = mm * ora_law_f64(law, rsm, r2);
        for (int q = 0; q < 3; ++q) a[q] += wg * d[q];
      }
      for (int q = 0; q < 3; ++q) dv[3 * i + q] += c * a[q];
    }
  }
  free(tab);
  free(tcut);
}

void ora_kick64_vjp(int64_t n, const double *pos, const double *m, int64_t nslots,
                    const int64_t *pnode_off, const int64_t *pnode_cnt, int law, double rsm,
                    double fsrrmax, double c, int64_t nleaves, const int64_t *leaf_offset,
                    const int64_t *leaf_count, const int64_t *list_ptr, const int64_t *list_idx,
                    const double *u, double *xbar) {
  double rmax2 = fsrrmax * fsrrmax;
  int64_t ntab = n + nslots;
  double *tab = (double *)malloc((size_t)(4 * ntab + 4) * sizeof(double));
  double *xt = (double *)calloc((size_t)(3 * ntab + 3), sizeof(double));
  tab64_fill(n, pos, m, nslots, pnode_off, pnode_cnt, tab);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t l = 0; l < nleaves; ++l) {
    for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i) {
      const double *ui = u + 3 * i;
      double acc[3] = {0, 0, 0};
      for (int64_t k = list_ptr[l]; k < list_ptr[l + 1]; ++k) {
        int64_t e = list_idx[k];
        if (e == i) continue;
        double d[3] = {tab[4 * e] - tab[4 * i], tab[4 * e + 1] - tab[4 * i + 1],
                       tab[4 * e + 2] - tab[4 * i + 2]};
        double wg, wgp;
        if (!pair_terms(law, rsm, rmax2, tab[4 * i + 3], tab[4 * e + 3], d, &wg, &wgp)) continue;
        double du = d[0] * ui[0] + d[1] * ui[1] + d[2] * ui[2];
        for (int a = 0; a < 3; ++a) {
          double v = c * (wg * ui[a] + 2.0 * wgp * du * d[a]);
          acc[a] -= v;
#ifdef _OPENMP
#pragma omp atomic
#endif
          xt[3 * e + a] += v;
        }
      }
      for (int a = 0; a < 3; ++a) {
#ifdef _OPENMP
#pragma omp atomic
#endif
        xt[3 * i + a] += acc[a];
      }
    }
  }
  for (int64_t k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) xbar[3 * k + a] += xt[3 * k + a];
  for (int64_t t = 0; t < nslots; ++t) {
    const double *g = xt + 3 * (n + t);
    double M = tab[4 * (n + t) + 3];
    if (M == 0 || (g[0] == 0 && g[1] == 0 && g[2] == 0)) continue;
    for (int64_t k = pnode_off[t]; k < pnode_off[t] + pnode_cnt[t]; ++k)
      for (int a = 0; a < 3; ++a) xbar[3 * k + a] += m[k] / M * g[a];
  }
  free(xt);
  free(tab);
}

typedef struct occ_t { int64_t leaf, pos; } occ_t;

void ora_fd_fp64_tab(int64_t n, const float *tab, int64_t ntab, const int64_t *pnode_off,
                     const int64_t *pnode_cnt, int law, float rsm, float fsrrmax, double c,
                     int64_t nleaves, const int64_t *leaf_offset, const int64_t *leaf_count,
                     const int64_t *list_ptr, const int64_t *list_idx, const double *u,
                     int64_t nsamples, const int64_t *samples, double h, double *fd, int32_t *near) {
  double rmax2 = (double)(fsrrmax * fsrrmax), rmax = sqrt(rmax2);
  /* occurrences of each sample as an entry, directly or through a pseudo-particle */
  int64_t *sample_of = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t k = 0; k < n; ++k) sample_of[k] = -1;
  for (int64_t s = 0; s < nsamples; ++s) sample_of[samples[s]] = s;
  occ_t **occ = (occ_t **)calloc((size_t)nsamples, sizeof(occ_t *));
  int64_t *nocc = (int64_t *)calloc((size_t)nsamples, sizeof(int64_t));
  int64_t *cap = (int64_t *)calloc((size_t)nsamples, sizeof(int64_t));
  int64_t *own = (int64_t *)malloc((size_t)(nsamples > 0 ? nsamples : 1) * sizeof(int64_t));
  for (int64_t s = 0; s < nsamples; ++s) own[s] = -1;
  for (int64_t l = 0; l < nleaves; ++l) {
    for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i)
      if (sample_of[i] >= 0) own[sample_of[i]] = l;
    for (int64_t pos = list_ptr[l]; pos < list_ptr[l + 1]; ++pos) {
      int64_t e = list_idx[pos];
      int64_t lo, hi;
      if (e < n) { lo = e; hi = e + 1; }
      else { lo = pnode_off[e - n]; hi = lo + pnode_cnt[e - n]; }
      for (int64_t s = 0; s < nsamples; ++s) {
        int64_t k = samples[s];
        if (k < lo || k >= hi) continue;
        if (nocc[s] == cap[s]) {
          cap[s] = cap[s] ? 2 * cap[s] : 64;
          occ[s] = (occ_t *)realloc(occ[s], (size_t)cap[s] * sizeof(occ_t));
        }
        occ[s][nocc[s]].leaf = l;
        occ[s][nocc[s]].pos = pos;
        nocc[s]++;
      }
    }
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t s = 0; s < nsamples; ++s) {
    int64_t k = samples[s];
    double mk = tab[4 * k + 3];
    near[s] = 0;
    for (int dim = 0; dim < 3; ++dim) {
      double Ls[2] = {0, 0};
      for (int sg = 0; sg < 2; ++sg) {
        double step = sg == 0 ? h : -h;
        double L = 0;
        /* position of table entry e with k displaced */
#define ENTRY_POS(e, out)                                                            \
  do {                                                                               \
    (out)[0] = tab[4 * (e)]; (out)[1] = tab[4 * (e) + 1]; (out)[2] = tab[4 * (e) + 2]; \
    if ((e) == k) (out)[dim] += step;                                                \
    else if ((e) >= n && k >= pnode_off[(e) - n] &&                                  \
             k < pnode_off[(e) - n] + pnode_cnt[(e) - n] && tab[4 * (e) + 3] != 0)   \
      (out)[dim] += step * mk / (double)tab[4 * (e) + 3];                            \
  } while (0)
        if (own[s] >= 0) { /* terms with i = k */
          int64_t l = own[s];
          double xk[3] = {tab[4 * k], tab[4 * k + 1], tab[4 * k + 2]};
          xk[dim] += step;
          for (int64_t pos = list_ptr[l]; pos < list_ptr[l + 1]; ++pos) {
            int64_t e = list_idx[pos];
            if (e == k) continue;
            double pe[3];
            ENTRY_POS(e, pe);
            double d[3] = {pe[0] - xk[0], pe[1] - xk[1], pe[2] - xk[2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (fabs(r - rmax) < 2 * h) near[s] = 1;
            double wg, wgp;
            if (!pair_terms(law, rsm, rmax2, mk, tab[4 * e + 3], d, &wg, &wgp)) continue;
            L += c * wg * (u[3 * k] * d[0] + u[3 * k + 1] * d[1] + u[3 * k + 2] * d[2]);
          }
        }
        for (int64_t q = 0; q < nocc[s]; ++q) { /* terms where k is (in) the entry */
          int64_t l = occ[s][q].leaf, pos = occ[s][q].pos, e = list_idx[pos];
          double pe[3];
          ENTRY_POS(e, pe);
          for (int64_t i = leaf_offset[l]; i < leaf_offset[l] + leaf_count[l]; ++i) {
            if (i == k || i == e) continue;
            double d[3] = {pe[0] - tab[4 * i], pe[1] - tab[4 * i + 1], pe[2] - tab[4 * i + 2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (fabs(r - rmax) < 2 * h) near[s] = 1;
            double wg, wgp;
            if (!pair_terms(law, rsm, rmax2, tab[4 * i + 3], tab[4 * e + 3], d, &wg, &wgp)) continue;
            L += c * wg * (u[3 * i] * d[0] + u[3 * i + 1] * d[1] + u[3 * i + 2] * d[2]);
          }
        }
#undef ENTRY_POS
        Ls[sg] = L;
      }
      fd[3 * s + dim] = (Ls[0] - Ls[1]) / (2 * h);
    }
  }
  for (int64_t s = 0; s < nsamples; ++s) free(occ[s]);
  free(occ);
  free(nocc);
  free(cap);
  free(own);
  free(sample_of);
}

/* ------------------------------------------------------------------------- */
/* Sub-cycle helpers (src/cpu/Particles.cxx)                                 */
/* ------------------------------------------------------------------------- */

void ora_map1(int64_t n, float *x, float *y, float *z, const float *vx, const float *vy,
              const float *vz, float alpha, float pp, float tau, float adot) {
  const float pf = powf(pp, (float)(1.0 + 1.0 / alpha));
  const float prefactor = (float)(1.0 / (alpha * adot * pf));
  for (int64_t i = 0; i < n; ++i) {
    x[i] = x[i] + prefactor * tau * vx[i];
    y[i] = y[i] + prefactor * tau * vy[i];
    z[i] = z[i] + prefactor * tau * vz[i];
  }
}

int64_t ora_resort(int64_t n, const int ng[3], float *x, float *y, float *z, float *vx,
                   float *vy, float *vz, float *phi, float *mass, int64_t *id,
                   uint16_t *mask) {
  int64_t Ng = (int64_t)ng[0] * ng[1] * ng[2];
  int64_t *cnt = (int64_t *)calloc((size_t)(Ng + 1), sizeof(int64_t));
  int64_t *cellof = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t *perm = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    int xx = (int)floorf(x[i]), yy = (int)floorf(y[i]), zz = (int)floorf(z[i]);
    int64_t c = (xx >= 0 && xx < ng[0] && yy >= 0 && yy < ng[1] && zz >= 0 && zz < ng[2])
                    ? ((int64_t)xx * ng[1] + yy) * ng[2] + zz
                    : Ng;
    cellof[i] = c;
    cnt[c]++;
  }
  int64_t inbox = n - cnt[Ng];
  int64_t run = 0;
  for (int64_t c = 0; c <= Ng; ++c) { int64_t t = cnt[c]; cnt[c] = run; run += t; }
  for (int64_t i = 0; i < n; ++i) perm[i] = cnt[cellof[i]]++;
  float *tmp = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  float *arrs[8] = {x, y, z, vx, vy, vz, phi, mass};
  for (int a = 0; a < 8; ++a) {
    for (int64_t i = 0; i < n; ++i) tmp[perm[i]] = arrs[a][i];
    memcpy(arrs[a], tmp, (size_t)n * sizeof(float));
  }
  int64_t *ti = (int64_t *)tmp;
  for (int64_t i = 0; i < n; ++i) ti[perm[i]] = id[i];
  memcpy(id, ti, (size_t)n * sizeof(int64_t));
  uint16_t *tm = (uint16_t *)tmp;
  for (int64_t i = 0; i < n; ++i) tm[perm[i]] = mask[i];
  memcpy(mask, tm, (size_t)n * sizeof(uint16_t));
  free(tmp);
  free(perm);
  free(cellof);
  free(cnt);
  return inbox;
}
