/*
 * hacc_sr.h -- C ABI of the GB300 short-range gravity path (RCBForceTree).
 *
 * This library replaces HACC's RCB force tree hot path: the tree build over a
 * rank's particles, the per-leaf interaction lists and the polynomial
 * short-range force law evaluated over every (leaf particle, list entry)
 * pair, fused with the sub-cycle velocity kick.  The pair evaluation runs as
 * hand-written CUDA kernels for sm_103a in FP32 on the CUDA cores.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   hsr_rcb_kick      <- template<int TDPTS> RCBForceTree::RCBForceTree(...)
 *                        src/halo_finder/RCBForceTree.h:96-124,
 *                        src/halo_finder/RCBForceTree.cxx:336-450
 *                        (build + list walk + nbody1 kick in one call)
 *   hsr_subcycle      <- Particles::subCycle / map1 / map2
 *                        src/cpu/Particles.cxx:1176-1201, 732-758, 1205-1367
 *   hsr_force_law     <- ForceLawSR::f_over_r over FGridEvalPoly
 *                        src/halo_finder/ForceLaw.cxx:137-141, 187-192
 *
 * Conventions: plain pointers and sizes only.  Particle arrays are the
 * reference's SoA layout (POSVEL_T = float, ID_T = int64_t, MASK_T = uint16_t,
 * src/halo_finder/BasicDefinition.h:60-91).  Every call returns an hsr_status;
 * where the reference calls exit(1) or assert()s (tree reallocation during a
 * parallel build, interaction list overflow), this library has no such limit
 * and returns HSR_OK.  One context per host thread; a context owns its CUDA
 * stream, device buffers and pinned staging memory.
 */
#ifndef HACC_SR_H
#define HACC_SR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t hsr_status;
enum {
  HSR_OK = 0,
  HSR_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, ...)   */
  HSR_ERR_CUDA = 2,         /* a CUDA runtime call failed (see hsr_last_error)  */
  HSR_ERR_NOMEM = 3,        /* host or device allocation failed                 */
  HSR_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up               */
  HSR_ERR_UNSUPPORTED = 5,  /* option combination not implemented               */
  HSR_ERR_NO_DEVICE = 6,    /* no CUDA device / the library's kernels cannot run */
  HSR_ERR_STATE = 7         /* call out of order (e.g. VJP before forward)      */
};

/* Where the particle arrays live. */
enum { HSR_MEM_HOST = 0, HSR_MEM_DEVICE = 1 };

/* Force laws.  POLY6: ForceLawSR over FGridEvalPoly, POLY_ORDER 6
 * (src/halo_finder/ForceLaw.cxx:93-141,187-192): g(r2) = (r2+rsm^2)^-3/2 -
 * sum_k a_k r2^k, with the pair weight m_i m_j.  POLY5_STEP16: the BG/Q
 * kernel Step16_int (src/halo_finder/BGQStep16.c:23-189): 5th-order
 * polynomial, weight m_j only, pairs with r2 == 0 dropped. */
enum { HSR_LAW_POLY6 = 0, HSR_LAW_POLY5_STEP16 = 1 };

/* Where the tree and the interaction lists are built (same results, bit for
 * bit).  DEVICE is the default. */
enum { HSR_BUILD_DEVICE = 0, HSR_BUILD_HOST = 1 };

/* Kernel variants for the pair evaluation (same results up to FP32
 * summation order). */
enum {
  HSR_KERNEL_AUTO = 0,      /* the context's tuned kernel (batched by default) */
  HSR_KERNEL_PLAIN = 1,     /* one CTA per leaf, every list entry evaluated    */
  HSR_KERNEL_BATCHED = 2    /* persistent CTAs over a work queue of tiles       */
};

/* RCBForceTree constructor arguments (src/halo_finder/RCBForceTree.h:96-124).
 * ForceLaw *fl is replaced by `law` + `rsm` (the law's softening). */
typedef struct hsr_params {
  float min[3], max[3];             /* minLoc, maxLoc: root bounding box        */
  float min_force[3], max_force[3]; /* minForceLoc, maxForceLoc                 */
  float avg_mass;                   /* avgMass (accepted, unused as in the ref) */
  float fsrrmax;                    /* fsm: cutoff radius                       */
  float rsm;                        /* softening of the force law               */
  float open_angle;                 /* oa, radians                              */
  int64_t nd;                       /* leaf size                                */
  int64_t ds;                       /* depth safety (accepted, unused)          */
  int64_t tmin;                     /* task size (accepted, unused)             */
  float fcoeff;                     /* kick coefficient                         */
  float ppc;                        /* pseudo-particle contraction factor       */
  int32_t tdpts;                    /* 1 = monopole, 12 = quadrupole            */
  int32_t law;                      /* HSR_LAW_*                                */
  int32_t kernel;                   /* HSR_KERNEL_*                             */
  int32_t build;                    /* HSR_BUILD_*                              */
  int32_t tree;                     /* HSR_TREE_* (0 = RCB)                     */
  int32_t reserved;                 /* 0                                        */
} hsr_params;

/* Tree kinds.  HSR_TREE_RCB is RCBForceTree (binary splits along the longest
 * axis at the centre of mass, src/halo_finder/RCBForceTree.cxx:778-890).
 * HSR_TREE_RCO is RCOForceTree (src/halo_finder/RCOForceTree.cxx:580-738: up
 * to eight children, all three axes split at the centre of mass), selected by
 * HACC's -O option (src/cpu/Particles.cxx:1259-1310); its tree and lists are
 * built on the host (hsr_rcb_kick with host arrays, hsr_build_lists), the
 * pairs on the device.  The reference's RCO partition reads past its 7-entry
 * split array (RCOForceTree.cxx:607-608); this library uses the end of the
 * processed range there, the value that makes the partition valid. */
enum { HSR_TREE_RCB = 0, HSR_TREE_RCO = 1 };

/* Statistics of the last call on a context. */
typedef struct hsr_stats {
  int64_t n;                 /* particles in the tree                           */
  int64_t nodes;             /* tree nodes                                      */
  int64_t leaves;            /* non-empty leaves                                */
  int64_t processed_leaves;  /* leaves inside the force box                     */
  int64_t list_entries;      /* sum of list lengths (self included)             */
  int64_t pairs;             /* sum over processed leaves of count * list length */
  int64_t kernel_launches;   /* CUDA kernels this call launched                 */
  double t_build_ms;         /* tree build (host: wall; device: events)         */
  double t_walk_ms;          /* interaction lists and work items (same)         */
  double t_force_ms;         /* device: pair kernel, CUDA events                */
  double t_total_ms;         /* wall time of the whole call                     */
  int64_t h2d_bytes;         /* bytes copied host -> device by the call         */
  int64_t d2h_bytes;         /* bytes copied device -> host by the call         */
  int64_t evaluated_pairs;   /* (particle, entry) pairs the kernel evaluated.
                                Device-built lists reach the kernels without
                                the entries farther than the cutoff from their
                                leaf's box (they contribute exactly 0): the
                                plain kernel evaluates every remaining entry
                                for each lane of a warp, the batched kernel
                                those that also pass its group's box test */
  int64_t work_items;        /* batched-kernel work items (group x list chunk)  */
  int64_t cm_fallbacks;      /* device build: nodes whose centre of mass needed
                                the sequential sum (see rcb_device.cuh)         */
  double t_h2d_ms;           /* device build: host -> device copies             */
  double t_d2h_ms;           /* device build: results back to the caller        */
} hsr_stats;

typedef struct hsr_ctx hsr_ctx;

/* Creates a context on CUDA device `device` (its own stream and buffers).
 * No counterpart in the reference (its tree is built per call with no
 * device state). */
hsr_status hsr_create(hsr_ctx **ctx, int device);
hsr_status hsr_destroy(hsr_ctx *ctx);
/* Message of the last error on this context (static storage, never NULL). */
const char *hsr_last_error(const hsr_ctx *ctx);
/* Library version string. */
const char *hsr_version(void);

/* The RCBForceTree constructor: builds the RCB tree over the n particles
 * (permuting all ten arrays in place exactly as the reference does), builds
 * the interaction list of every leaf inside the force box and adds
 * fcoeff * sum_j m_i m_j g(r2_ij) (x_j - x_i) to v_i for r2_ij < fsrrmax^2.
 * mem: HSR_MEM_HOST (any host memory) or HSR_MEM_DEVICE (device pointers on
 * the context's device; HSR_BUILD_DEVICE only).  Synchronous: the arrays
 * hold the result when the call returns.  Replaces the constructor
 * RCBForceTree<TDPTS>::RCBForceTree (src/halo_finder/RCBForceTree.h:96-124,
 * src/halo_finder/RCBForceTree.cxx:336-450). */
hsr_status hsr_rcb_kick(hsr_ctx *ctx, const hsr_params *p, int64_t n, float *x, float *y,
                        float *z, float *vx, float *vy, float *vz, float *mass, float *phi,
                        int64_t *id, uint16_t *mask, int32_t mem);

hsr_status hsr_get_stats(const hsr_ctx *ctx, hsr_stats *st);

/* Several independent boxes in one call (multi-box batching; no
 * counterpart in the reference, which kicks one rank's box per constructor):
 * every box's tree and lists are built on the device (up to four boxes at
 * once, each on its own stream and host thread), then ONE persistent
 * launch of the batched kernel evaluates the work items of all boxes, each
 * with its own parameters (fcoeff, rsm, cutoff; one force law for all).  The
 * per-box arrays are given as arrays of nbox pointers; each box's arrays are
 * permuted and kicked exactly as hsr_rcb_kick would.  Statistics sum over the
 * boxes. */
hsr_status hsr_rcb_kick_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                              const int64_t *n, float *const *x, float *const *y,
                              float *const *z, float *const *vx, float *const *vy,
                              float *const *vz, float *const *mass, float *const *phi,
                              int64_t *const *id, uint16_t *const *mask, int32_t mem);

/* Interaction lists of the last hsr_rcb_kick, for inspection and parity
 * checks.  hsr_lists_size gives the number of processed leaves and of list
 * entries; hsr_lists_export fills leaf_offset/leaf_count (per leaf, into the
 * permuted arrays), list_ptr (nleaves+1) and the entries as the reference's
 * nx/ny/nz/nm arrays would hold them (any order within a leaf).  No call
 * of the reference returns them: they are the lists calcInternodeForce
 * builds on its stack (src/halo_finder/RCBForceTree.cxx:923-1144, arrays
 * declared at :940). */
hsr_status hsr_lists_size(const hsr_ctx *ctx, int64_t *nleaves, int64_t *nentries);
hsr_status hsr_lists_export(const hsr_ctx *ctx, int64_t *leaf_offset, int64_t *leaf_count,
                            int64_t *list_ptr, float *ex, float *ey, float *ez, float *em);

/* Host-only tree build and interaction lists, no device work: the same tree,
 * permutation and lists as hsr_rcb_kick (the ten arrays are permuted in
 * place, velocities are not kicked), kept in a standalone handle.  Replaces
 * the build and list halves of the RCBForceTree constructor
 * (src/halo_finder/RCBForceTree.cxx:892-918, 923-1197) for callers that
 * evaluate the pairs themselves; also what the CPU test suite uses to check
 * the lists without a GPU. */
typedef struct hsr_lists hsr_lists;
hsr_status hsr_build_lists(const hsr_params *p, int64_t n, float *x, float *y, float *z,
                           float *vx, float *vy, float *vz, float *mass, float *phi, int64_t *id,
                           uint16_t *mask, hsr_lists **out);
/* nleaves/nentries as hsr_lists_size; stats as hsr_get_stats (no timings of
 * device work).  Accessors of hsr_build_lists' result: the lists of
 * src/halo_finder/RCBForceTree.cxx:923-1144. */
hsr_status hsr_lists_info(const hsr_lists *L, int64_t *nleaves, int64_t *nentries, hsr_stats *st);
hsr_status hsr_lists_get(const hsr_lists *L, int64_t *leaf_offset, int64_t *leaf_count,
                         int64_t *list_ptr, float *ex, float *ey, float *ez, float *em);
/* Position-table index of every entry: < n is a particle (post-permutation
 * index), >= n a pseudo-particle.  (The list entries of
 * src/halo_finder/RCBForceTree.cxx:1129-1139 and :1085-1123, named by
 * where they come from.) */
hsr_status hsr_lists_index(const hsr_lists *L, int64_t *entry_index);
hsr_status hsr_lists_free(hsr_lists *L);

/* ---- launch shapes ------------------------------------------------------ */

/* Launch shape of the pair kernels, held per context.  Kicks with
 * HSR_KERNEL_AUTO run `kernel`; the plain kernel runs `leaf_threads` threads
 * per leaf (32, 64 or 128); the batched kernel takes work items of `group`
 * particles (16 or 32).  Defaults: HSR_KERNEL_BATCHED, 128, 32.  The shape
 * changes the FP32 summation order only, never the pair set.  No counterpart in
 * the reference (nbody1, src/halo_finder/RCBForceTree.cxx:575-620, is a plain
 * loop with no launch shape). */
typedef struct hsr_tune {
  int32_t kernel;        /* HSR_KERNEL_PLAIN or HSR_KERNEL_BATCHED */
  int32_t leaf_threads;  /* 32, 64, 128 */
  int32_t group;         /* 16, 32 */
  int32_t reserved;      /* 0 */
} hsr_tune;

typedef struct hsr_tune_row {
  hsr_tune tune;
  double ms;                /* mean device time of one pair-kernel launch */
  int64_t evaluated_pairs;  /* pairs the launch evaluated */
} hsr_tune_row;

hsr_status hsr_set_tune(hsr_ctx *ctx, const hsr_tune *t);
hsr_status hsr_get_tune(const hsr_ctx *ctx, hsr_tune *t);

/* Times every shape (plain kernel with 32, 64 and 128 threads per leaf,
 * batched kernel with groups of 16 and 32) on the tree and lists of the last
 * single-box kick built on the device, `iters` launches each after one
 * warm-up launch (L2 flushed before each when flush_l2 != 0), and sets the
 * context's shape to the fastest.  The launches accumulate into the context's
 * own velocity scratch, never into caller arrays.  Writes min(cap, *nrows)
 * rows; *nrows receives the number of shapes timed.  HSR_ERR_STATE without
 * such a kick.  No counterpart in the reference (its nbody1 has one fixed
 * loop shape). */
hsr_status hsr_autotune(hsr_ctx *ctx, int32_t iters, int32_t flush_l2, hsr_tune_row *rows,
                        int32_t cap, int32_t *nrows);

/* ---- the sub-cycle around the kick ------------------------------------- */

/* Particles::subCycle (src/cpu/Particles.cxx:1176-1201) with map1 (:732-758)
 * and map2 (:1205-1367) on the device: nsub times
 *   half-stream  x += prefactor * tau * v,
 *   resort       stable sort by unit grid cell of the ng box, out-of-box last,
 *   masses = 1,
 *   kick         the RCB short-range kick (hsr_rcb_kick) of the in-box
 *                particles with `kick` (fcoeff = map2's c),
 *   half-stream.
 * prefactor = 1 / (alpha * adot * pp^(1 + 1/alpha)) in float as map1 computes
 * it; tau is map1's argument (stepFraction * tau2).  The arrays stay resident
 * on the device for all sub-cycles.  *n_inbox receives the in-box count of the
 * last resort. */
typedef struct hsr_subcycle_params {
  hsr_params kick;
  int32_t nsub;
  int32_t ng[3];
  float alpha, pp, tau, adot;
  int32_t skip_stream, skip_kick;
} hsr_subcycle_params;

hsr_status hsr_subcycle(hsr_ctx *ctx, const hsr_subcycle_params *sp, int64_t n, float *x,
                        float *y, float *z, float *vx, float *vy, float *vz, float *mass,
                        float *phi, int64_t *id, uint16_t *mask, int32_t mem, int64_t *n_inbox);

/* ---- adjoint (vector-Jacobian product) --------------------------------- */

/* Forward half: the short-range velocity change the kick would apply,
 *   dv_i = fcoeff m_i sum_{j in list(i), r2 < fsrrmax^2} m_j g(r2) (x_j - x_i)
 * (zero for particles outside the processed leaves), for positions x, y, z and
 * masses (read only, never permuted), written to dvx, dvy, dvz in the
 * caller's order.  Keeps the tree, lists and positions on the context as the
 * tape for hsr_force_vjp (any other kick or forward call replaces it).
 * mem: HSR_MEM_HOST or HSR_MEM_DEVICE; the tree is built on the device.
 * No counterpart in the reference (differentiation is new in this library). */
hsr_status hsr_force_fwd(hsr_ctx *ctx, const hsr_params *p, int64_t n, const float *x,
                         const float *y, const float *z, const float *mass, float *dvx,
                         float *dvy, float *dvz, int32_t mem);

/* hsr_force_fwd that adds dv into (vx, vy, vz), the caller's order, instead
 * of writing it: the sub-cycle's short-range kick (RCBForceTree's nbody1
 * update v += fcoeff m_i sum_j m_j g d, src/halo_finder/RCBForceTree.cxx:
 * 599-619) without permuting the caller's arrays, so a multi-step driver
 * keeps every particle at a fixed index.  Records the same tape as
 * hsr_force_fwd. */
hsr_status hsr_force_kick(hsr_ctx *ctx, const hsr_params *p, int64_t n, const float *x,
                          const float *y, const float *z, const float *mass, float *vx,
                          float *vy, float *vz, int32_t mem);

/* Several independent boxes of the forward half at once (multi-box batching;
 * no counterpart in the reference, which kicks one rank's box per
 * RCBForceTree constructor): every box's tree and lists are built on the
 * device (boxes prepared concurrently, each on its own stream), then ONE
 * persistent launch of the pair kernel evaluates the work items of all boxes
 * (a CUDA graph, captured on each call and replayed through the context's
 * executable graph), each box with its own parameters (one force law for
 * all).  Per box as hsr_force_fwd: positions and masses are read only, dv is
 * written in the caller's order; arrays are given as arrays of nbox
 * pointers.  The boxes' trees and lists stay on the context as the tape of
 * hsr_force_vjp_batch (any other kick or forward call replaces it).
 * Statistics sum over the boxes. */
hsr_status hsr_force_fwd_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                               const int64_t *n, const float *const *x, const float *const *y,
                               const float *const *z, const float *const *mass, float *const *dvx,
                               float *const *dvy, float *const *dvz, int32_t mem);

/* hsr_force_fwd_batch that adds every box's dv into its (vx, vy, vz) (the
 * caller's order) instead of writing it: one sub-cycle kick of several boxes
 * in one persistent launch, as hsr_force_kick is for one box (one
 * RCBForceTree kick, src/halo_finder/RCBForceTree.cxx:599-619, per box). */
hsr_status hsr_force_kick_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                                const int64_t *n, const float *const *x, const float *const *y,
                                const float *const *z, const float *const *mass, float *const *vx,
                                float *const *vy, float *const *vz, int32_t mem);

/* Backward half of hsr_force_fwd_batch / hsr_force_kick_batch: for every box,
 * xbar_b = (d dv_b / d x_b)^T dvbar_b over the tape of the last multi-box
 * forward (nbox must equal its box count), caller's order, the VJP of all
 * boxes in one persistent launch.  As hsr_force_vjp: trees, lists and the
 * cutoff held fixed, monopole or 12-point pseudo-particles per box;
 * HSR_ERR_STATE without a multi-box forward.  No counterpart in the
 * reference (differentiation is new in this library). */
hsr_status hsr_force_vjp_batch(hsr_ctx *ctx, int32_t nbox, const float *const *dvbx,
                               const float *const *dvby, const float *const *dvbz,
                               float *const *xbx, float *const *xby, float *const *xbz,
                               int32_t mem);

/* Particles::map1 (src/cpu/Particles.cxx:732-758) on device arrays:
 * x += pt * v for the three components, pt = prefactor * tau with prefactor =
 * 1 / (alpha * adot * pp^(1 + 1/alpha)), all in float as map1 computes them.
 * Called with (vbar, xbar) in place of (x, v) it is also the half-stream's adjoint
 * (vbar += pt xbar).  mem must be HSR_MEM_DEVICE. */
hsr_status hsr_stream(hsr_ctx *ctx, int64_t n, float *x, float *y, float *z, const float *vx,
                      const float *vy, const float *vz, float alpha, float pp, float tau,
                      float adot, int32_t mem);

/* Backward half: xbar = (d dv / d x)^T dvbar for the tape of the last
 * hsr_force_fwd, caller's order, with the tree and the lists held fixed (they
 * are piecewise constant in the positions).  A monopole pseudo-particle sits
 * at its node's centre of mass, so its gradient passes on to the node's
 * particles with weights m_k / M_node.  12-point pseudo-particles
 * (RCBForceTree.cxx:519-568): their positions and masses depend on the
 * node's sources, centre of mass and tdr; the gradient passes through all of
 * them, top down (tdr's to the particle on the box face it is measured to).
 * The cutoff is a step: its delta contribution is not included.
 * HSR_ERR_STATE without a forward. */
hsr_status hsr_force_vjp(hsr_ctx *ctx, const float *dvbx, const float *dvby, const float *dvbz,
                         float *xbx, float *xby, float *xbz, int32_t mem);

/* The tree order of the last kick or forward: position k holds input
 * particle perm[k] (n entries): the permutation the reference's partition
 * applies to the ten arrays in place (src/halo_finder/RCBForceTree.cxx:
 * 623-672), for callers that keep particles at fixed indices. */
hsr_status hsr_last_perm(const hsr_ctx *ctx, int64_t *perm);

/* The last tree's nodes (any numbering; children have larger indices than
 * their parents): particle range, children (0 = none), pseudo-particle
 * radius, box and centre of mass (xmin[3], xmax[3], xc[3] per node) and the
 * tdpts pseudo-particle masses per node.  A node's pseudo-particles sit at
 * position-table index n + node * tdpts.  The reference keeps these as its
 * TreeNode vector (src/halo_finder/RCBForceTree.h:131-147) without an
 * accessor. */
hsr_status hsr_tree_size(const hsr_ctx *ctx, int64_t *nnodes);
hsr_status hsr_tree_export(const hsr_ctx *ctx, int64_t *count, int64_t *offset, int64_t *cl,
                           int64_t *cr, float *tdr, float *bbox9, float *ppm);

/* Position-table index of every list entry of the last kick or forward, in
 * the order of hsr_lists_export (< n: particle in tree order, >= n:
 * pseudo-particle); the entries of src/halo_finder/RCBForceTree.cxx:
 * 1085-1139 named by where they come from. */
hsr_status hsr_lists_export_index(const hsr_ctx *ctx, int64_t *entry_index);

/* ForceLawSR::f_over_r on the device for a batch of r2 values (host arrays),
 * with the kernel's own FP32 arithmetic; for law tests.  Replaces
 * ForceLawSR::f_over_r over FGridEvalPoly::eval
 * (src/halo_finder/ForceLaw.cxx:137-141, 187-192). */
hsr_status hsr_force_law(hsr_ctx *ctx, int32_t law, float rsm, float fsrrmax, int64_t n,
                         const float *r2, float *g);

/* The short-range kick over interaction lists the caller already holds on the
 * device, with no memory allocation of any kind.  No counterpart in the
 * reference.
 *
 * For callers that cannot allocate device memory once running (a simulation
 * that sizes all buffers at start-up and forbids allocation in its time loop,
 * code whose memory pool or arena owns the device, an embedding that must not
 * grow its footprint).  Everything is the caller's: the position table
 * (ntab entries of 4 floats x, y, z, m, 16-byte aligned; entries >= n are
 * pseudo-particles), the leaves (particle offset and count, list begin and
 * length, as hsr_lists_export / hsr_build_lists describe them), the list
 * entries as table indices, and vx, vy, vz (n floats, kicked in place, in
 * table order) -- all device pointers on the current device.  The kernel's
 * scratch (work items and counters) lives in a fixed 4 MiB device array that
 * every device loading the library holds until the process exits; lists that
 * need more than 131064 work items (one per group of up to 32 leaf particles
 * per 8192 list entries) are rejected with HSR_ERR_ARG and no pair is
 * evaluated (the velocities are left as they were).  The first call on a
 * device looks up that array's device address (set-up); make that first call
 * before any stream capture.  Later calls look the address up again unless
 * their stream is capturing.  Calls share the array, which keeps the last
 * call's contents (each call clears its counters first): calls that overlap
 * on the GPU race and must not be issued concurrently.  `stream` (NULL: the
 * default stream) must belong to the current device, else HSR_ERR_ARG.  The
 * call returns after its work on the stream has finished: it synchronizes
 * the stream to read the overflow flag back. */
hsr_status hsr_kick_lists_noalloc(const float *table, int64_t ntab, int64_t n,
                                  const int32_t *leaf_offset, const int32_t *leaf_count,
                                  const int64_t *list_begin, const int32_t *list_len,
                                  int64_t nleaves, const int32_t *list_index, float *vx, float *vy,
                                  float *vz, float fcoeff, float rsm, float fsrrmax, int32_t law,
                                  void *stream);

/* ---- diagnostics ------------------------------------------------------- */

/* Relaunches the pair kernel of the last hsr_rcb_kick `iters` times on the
 * work still resident on the device (the velocities keep accumulating kicks),
 * each launch timed with CUDA events on the context's stream.  flush_l2 != 0
 * overwrites a 256 MB device buffer before every launch so no launch starts
 * with the previous one's data in L2.  *ms_per_launch is the mean time.
 * kernel: HSR_KERNEL_PLAIN or the kick's own; HSR_KERNEL_BATCHED after
 * hsr_rcb_kick_batch replays its one multi-box launch.  use_graph != 0 replays
 * the launch sequence (queue reset + kernel) as a captured CUDA graph.
 * Measurement only: no counterpart in the reference. */
hsr_status hsr_bench_pairs(hsr_ctx *ctx, int32_t kernel, int32_t iters, int32_t flush_l2,
                           double *ms_per_launch);
hsr_status hsr_bench_pairs_graph(hsr_ctx *ctx, int32_t iters, int32_t flush_l2,
                                 double *ms_per_launch);

/* The number of (leaf particle, list entry) pairs of the last single-box kick
 * built on the device whose distance is within the cutoff (r2 < the law's
 * cutoff squared, r2 rounded as the reference's nbody1 computes it): the
 * pairs that contribute, beside hsr_stats.pairs (every listed pair).
 * HSR_ERR_STATE without such a kick.  Measurement only: the reference's
 * nbody1 masks these pairs per term (src/halo_finder/RCBForceTree.cxx:
 * 612-617) without counting them. */
hsr_status hsr_pairs_in_cutoff(hsr_ctx *ctx, int64_t *count);

/* Measures this device's FP32 FMA throughput with a kernel of independent
 * fused multiply-add chains (2 flops each) on every SM; the roofline
 * denominator of the pair kernels.  Measurement only: no counterpart in the
 * reference. */
hsr_status hsr_probe_fp32_peak(hsr_ctx *ctx, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* HACC_SR_H */
