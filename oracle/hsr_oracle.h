/*
 * hsr_oracle.h -- CPU restatement of HACC's RCBForceTree short-range hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU library is
 * compared against and the CPU baseline it is timed beside.  It is never
 * linked into, loaded by or called from the product library; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Parity is pinned: on seeded inputs its outputs are compared bit for bit with
 * the reference sources compiled unmodified (oracle/Makefile builds
 * oracle/_ref/rcb_ref), and the fixtures in tests/golden/ were written by that
 * reference build (tests/golden/make_golden.py).
 *
 * Reference files are cited by their path inside the reference project.
 */
#ifndef HSR_ORACLE_H
#define HSR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Force laws.  POLY6 is ForceLawSR over FGridEvalPoly with POLY_ORDER 6
 * (src/halo_finder/ForceLaw.cxx:93-141,187-192), the law HACC's -P option and
 * this project use.  POLY5_STEP16 is the BG/Q kernel Step16_int
 * (src/halo_finder/BGQStep16.c:23-189): 5th-order polynomial, no m_i factor,
 * pairs with r2 == 0 dropped, arithmetic in double.  It cannot be run here (QPX),
 * so that mode is restated from the source and is not pinned. */
enum { ORA_LAW_POLY6 = 0, ORA_LAW_POLY5_STEP16 = 1 };

typedef struct ora_params {
  float min[3], max[3];             /* minLoc / maxLoc: root bounding box          */
  float min_force[3], max_force[3]; /* minForceLoc / maxForceLoc                   */
  float avg_mass;                   /* avgMass (stored, unused, as in the ref)     */
  float fsrrmax;                    /* fsm: short-range cutoff radius              */
  float rsm;                        /* softening length of the force law           */
  float open_angle;                 /* oa, radians                                 */
  int64_t nd;                       /* leaf size: nodes with count <= nd are leaves */
  int64_t ds;                       /* depth safety (capacity hint only)           */
  int64_t tmin;                     /* task threshold (unused by the sections build) */
  float fcoeff;                     /* kick coefficient                            */
  float ppc;                        /* pseudo-particle contraction factor          */
  int32_t tdpts;                    /* 1 = monopole, 12 = quadrupole               */
  int32_t law;                      /* ORA_LAW_*                                   */
  int32_t vmax;                     /* >0: fail like the reference when a list
                                       reaches this many entries (VMAX = 16384)    */
  int32_t nthreads;                 /* 0 = OpenMP default                          */
  int32_t tree;                     /* ORA_TREE_RCB or ORA_TREE_RCO                 */
} ora_params;

/* Tree kinds: RCBForceTree (binary splits along the longest axis) and
 * RCOForceTree (src/halo_finder/RCOForceTree.cxx: up to eight children split
 * along all three axes at the centre of mass). */
enum { ORA_TREE_RCB = 0, ORA_TREE_RCO = 1 };

typedef struct ora_stats {
  int64_t nodes;            /* tree nodes allocated (incl. unused split pairs)   */
  int64_t leaves;           /* leaves with count > 0                             */
  int64_t empty_leaves;
  int64_t max_ppn;
  int64_t processed_leaves; /* leaves inside the force box                       */
  int64_t list_entries;     /* sum of list lengths (self included)               */
  int64_t pairs;            /* sum over processed leaves of count * list length  */
  double t_build;           /* seconds, wall                                     */
  double t_walk;            /* seconds, wall: lists + force + kick               */
} ora_stats;

typedef struct ora_result ora_result;

/* The whole RCBForceTree constructor (src/halo_finder/RCBForceTree.cxx:336-450):
 * builds the tree (permuting all ten arrays in place), walks it and kicks
 * vx, vy, vz.  keep_lists != 0 stores every processed leaf's interaction list
 * for export.  do_kick == 0 builds the lists but leaves the velocities alone.
 * Returns NULL on bad arguments; *err receives an ORA_ERR_* code. */
enum { ORA_OK = 0, ORA_ERR_ARG = 1, ORA_ERR_VMAX = 2, ORA_ERR_NOMEM = 3 };

ora_result *ora_rcb_run(const ora_params *p, int64_t n,
                        float *x, float *y, float *z,
                        float *vx, float *vy, float *vz,
                        float *mass, float *phi, int64_t *id, uint16_t *mask,
                        int keep_lists, int do_kick, int *err);

void ora_result_stats(const ora_result *r, ora_stats *st);
int64_t ora_result_nleaves(const ora_result *r);
int64_t ora_result_nentries(const ora_result *r);
/* CSR export of the processed leaves in DFS order: leaf particle range and the
 * offsets of each leaf's list in the entry arrays (list_ptr has nleaves+1). */
void ora_result_leaves(const ora_result *r, int64_t *leaf_offset,
                       int64_t *leaf_count, int64_t *list_ptr);
/* Entries exactly as the reference's nx/ny/nz/nm arrays hold them. */
void ora_result_entries(const ora_result *r, float *ex, float *ey, float *ez,
                        float *em);
/* Tree node export (count, offset, cl, cr, tdr, xmin, xmax, xc, ppm[0..tdpts)). */
int64_t ora_result_nnodes(const ora_result *r);
void ora_result_nodes(const ora_result *r, int64_t *count, int64_t *offset,
                      int64_t *cl, int64_t *cr, float *tdr, float *bbox9,
                      float *ppm);
/* FP64 evaluation over the same lists: acceleration a_i = sum_j m_i m_j g(r2) d
 * (no fcoeff) for the particles of the processed leaves, written at their
 * post-permutation index.  Other entries are left untouched. */
void ora_result_acc_fp64(const ora_result *r, double *ax, double *ay, double *az);
void ora_result_free(ora_result *r);

/* Short-range law g(r2) = f_over_r(r2) in FP32 exactly as the reference
 * evaluates it, and its FP64 counterpart with the same coefficients. */
float ora_law_f32(int law, float rsm, float r2);
double ora_law_f64(int law, double rsm, double r2);
/* d g / d(r2) in FP64 (for adjoint checks). */
double ora_law_dg_f64(int law, double rsm, double r2);

/* FP64 direct sum over all n particles for the listed targets: a_t =
 * sum_{j, r2 < rmax^2} m_t m_j g(r2) d.  Cell-list accelerated. */
void ora_direct_fp64(int64_t n, const float *x, const float *y, const float *z,
                     const float *mass, int law, float rsm, float fsrrmax,
                     int64_t ntargets, const int64_t *targets,
                     double *ax, double *ay, double *az);

/* FP64 vector-Jacobian product of the pair force over fixed CSR lists of real
 * particles (list entries are particle indices).  For cotangent u (per
 * particle, 3 components), returns xbar = (d a / d x)^T u, where
 * a_i = c * sum_{j in list(i)} [r2 < rmax2] m_i m_j g(r2) (x_j - x_i). */
void ora_vjp_fp64(int64_t n, const float *x, const float *y, const float *z,
                  const float *mass, int law, float rsm, float fsrrmax, double c,
                  int64_t nleaves, const int64_t *leaf_offset,
                  const int64_t *leaf_count, const int64_t *list_ptr,
                  const int64_t *list_idx, const double *u, double *xbar);

/* The same VJP over lists of position-table indices (tab: ntab x 4 floats,
 * x y z m; entries >= n are monopole pseudo-particles at their node's centre
 * of mass, node particle range pnode_off/pnode_cnt per slot idx - n), with
 * self entries skipped: xbar = (d dv / d x)^T u for dv_i = c m_i sum_j m_j g d.
 * u, xbar: n x 3. */
void ora_vjp_fp64_tab(int64_t n, const float *tab, int64_t ntab, const int64_t *pnode_off,
                      const int64_t *pnode_cnt, int law, float rsm, float fsrrmax, double c,
                      int64_t nleaves, const int64_t *leaf_offset, const int64_t *leaf_count,
                      const int64_t *list_ptr, const int64_t *list_idx, const double *u,
                      double *xbar);
/* FP64 central differences of L = sum_i u_i . dv_i with the lists fixed, for
 * each sampled particle k (tree order) and axis: fd[3s + d].  near[s] = 1 when
 * a pair involving k lies within 2h of the cutoff (the law steps there). */
void ora_fd_fp64_tab(int64_t n, const float *tab, int64_t ntab, const int64_t *pnode_off,
                     const int64_t *pnode_cnt, int law, float rsm, float fsrrmax, double c,
                     int64_t nleaves, const int64_t *leaf_offset, const int64_t *leaf_count,
                     const int64_t *list_ptr, const int64_t *list_idx, const double *u,
                     int64_t nsamples, const int64_t *samples, double h, double *fd, int32_t *near);

/* FP64 kick over lists of table indices with positions in FP64 (pos: n x 3,
 * tree order; m: masses).  Table entries >= n are monopole pseudo-particles at
 * the FP64 centre of mass of their node's particles (node slot t = idx - n,
 * particle range pnode_off/pnode_cnt); self entries skipped.
 * dv (n x 3) += c m_i sum_j m_j g(r2) d over the cutoff.  pos_cut, when not
 * NULL, holds reference positions (n x 3) on which each pair's cutoff test is
 * made instead (the map with its cutoff mask frozen, for difference checks). */
void ora_kick64(int64_t n, const double *pos, const double *m, int64_t nslots,
                const int64_t *pnode_off, const int64_t *pnode_cnt, int law, double rsm,
                double fsrrmax, double c, int64_t nleaves, const int64_t *leaf_offset,
                const int64_t *leaf_count, const int64_t *list_ptr, const int64_t *list_idx,
                const double *pos_cut, double *dv);
/* Its vector-Jacobian product: xbar (n x 3) += (d dv / d pos)^T u, the
 * centre-of-mass chain rule included. */
void ora_kick64_vjp(int64_t n, const double *pos, const double *m, int64_t nslots,
                    const int64_t *pnode_off, const int64_t *pnode_cnt, int law, double rsm,
                    double fsrrmax, double c, int64_t nleaves, const int64_t *leaf_offset,
                    const int64_t *leaf_count, const int64_t *list_ptr, const int64_t *list_idx,
                    const double *u, double *xbar);

/* Particles::map1 (src/cpu/Particles.cxx:732-758): x += prefactor*tau*v. */
void ora_map1(int64_t n, float *x, float *y, float *z, const float *vx,
              const float *vy, const float *vz, float alpha, float pp,
              float tau, float adot);
/* Particles::resortParticles (src/cpu/Particles.cxx:402-488): stable counting
 * sort by grid cell, out-of-box particles last.  Returns the in-box count. */
int64_t ora_resort(int64_t n, const int ng[3], float *x, float *y, float *z,
                   float *vx, float *vy, float *vz, float *phi, float *mass,
                   int64_t *id, uint16_t *mask);

#ifdef __cplusplus
}
#endif
#endif
