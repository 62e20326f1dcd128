// rcb_device.cuh -- the RCB tree build, the interaction lists and the
// batched work description on the GPU.
//
// Reproduces the reference exactly (the same permutation of the particle
// arrays, the same centres of mass, bounding boxes, pseudo-particles and
// interaction lists) as the host implementation in rcb_host.cpp:
//   build  : src/halo_finder/RCBForceTree.cxx:623-918, src/halo_finder/BGQCM.c:181-212
//   lists  : src/halo_finder/RCBForceTree.cxx:923-1197
// Level by level, all nodes of a level at once:
//   * bounding box and centre of mass per node by a chunked segmented
//     reduction.  The reference sums the centre of mass in double in array
//     order; the parallel sum differs from it by at most a bound covering both
//     summation orders.  When both ends of that bound round to the same float,
//     that float is the reference's centre of mass; otherwise (rare, ~1e-2 of
//     the root's coordinates) one thread repeats the reference's sequential
//     sum for that node.
//   * the partition at the centre of mass: ranks of the "left" particles by a
//     scan; the reference's swap sequence moves each remaining particle along
//     a chain of left positions (p -> idx[p] -> ...), which one thread per
//     particle follows (chains average two steps).
// Every float expression that decides the tree or a list uses explicitly
// rounded intrinsics so no multiply-add is fused, as in the reference.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "sr_kernels.cuh"

namespace hsr {

// Tree node on the device (the reference's TreeNode, RCBForceTree.h:131-147).
struct alignas(16) DNode {
  int32_t count, offset, cl, cr;  // cl == cr == 0: leaf
  float xmin[3], xmax[3], xc[3], tdr;
  int32_t split_dim;              // -1: no split attempted (leaf by size)
  int32_t nleft;                  // particles below the split (partition result)
};

struct TreeConfig {
  float min[3], max[3], min_force[3], max_force[3];
  float fsrrmax, tan_oa, ppc;
  int32_t nd, tdpts;
  int32_t force_cm_fallback;  // test hook: 1 = every node takes the sequential sum,
                              // 2 = every node goes through the tight certification
  int32_t group;              // particles per work-item group: 16 or 32 (0 = 32)
  float prune2;               // > 0: the index lists keep only entries within
                              // sqrt(prune2) of their leaf's box (the kernels'
                              // cull radius); 0: every list entry
};

// Result sizes of a device build.
struct DeviceTreeInfo {
  int64_t nodes = 0, levels = 0, leaves = 0, processed_leaves = 0;
  int64_t segments = 0, list_entries = 0, pairs = 0, items = 0;
  int64_t cm_fallbacks = 0;
  int64_t launches = 0;  // kernels launched by the last build() and the item setups after it
};

// Owns the device buffers of one tree; reused across calls (grows only).
class DeviceTree {
 public:
  DeviceTree() = default;
  ~DeviceTree();
  DeviceTree(const DeviceTree &) = delete;
  DeviceTree &operator=(const DeviceTree &) = delete;

  // Builds the tree over n particles whose (x, y, z, m) are in `pos_in`
  // (float4, device).  Afterwards `perm()` maps each final position to its
  // input index, `table()` holds the position table (particles in tree order,
  // then tdpts pseudo-particles per node), and the processed leaves' lists,
  // work items and group index are built.  `jsplit` bounds the list range of
  // one work item.  Synchronizes `s` once per tree level down to the first
  // level whose nodes all fit one block; that level's subtrees are built
  // whole, one block each, with one synchronisation.
  cudaError_t build(const TreeConfig &cfg, int64_t n, const float4 *pos_in, int64_t jsplit,
                    cudaStream_t s);

  // Rebuilds the groups and work items of the last build for another group
  // size (16 or 32); the tree and the lists stay.
  cudaError_t regroup(int group, int64_t jsplit, cudaStream_t s);
  int group() const { return group_; }

  const DeviceTreeInfo &info() const { return info_; }
  const int32_t *perm() const { return oid_; }
  const float4 *table() const { return table_; }
  const LeafDesc *leaves() const { return leafdesc_; }
  const SegDesc *segs() const { return segs_; }
  const int32_t *index() const { return idx_list_; }
  const PairItem *items() const { return items_; }
  const int32_t *gidx() const { return gidx_; }
  const DNode *nodes() const { return nodes_; }
  const float *ppm() const { return ppm_; }
  // First node of each tree level (BFS order), plus the node count at the end.
  const std::vector<int32_t> &levels() const { return levels_; }
  const int32_t *leaf_nodes() const { return leaf_ids_; }
  int64_t padded_pairs() const { return padded_pairs_; }
  // Device time of the last build's tree levels and of its lists + items.
  double build_ms() const { return build_ms_; }
  double lists_ms() const { return lists_ms_; }
  // Whether a device-side bound was hit (walk stack); the build then failed.
  const char *error() const { return err_; }

 private:
  template <typename T>
  cudaError_t grow(T *&p, size_t &cap, size_t count, cudaStream_t s, bool keep = false);
  cudaError_t make_items(int64_t n, int64_t jsplit, cudaStream_t s);
  // exclusive_scan_i64, adding its kernels to info_.launches
  cudaError_t scan_counted(const int64_t *in, int64_t *out, int64_t n, int64_t *total, int64_t *tmp,
                           cudaStream_t s);

  DeviceTreeInfo info_{};
  int64_t padded_pairs_ = 0;
  double build_ms_ = 0, lists_ms_ = 0;
  std::vector<int32_t> levels_;
  const char *err_ = nullptr;
  int group_ = 32;
  // the build's groups run on their own stream beside the list walk
  cudaStream_t aux_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_groups_ = nullptr;
  int groups_ready_ = 0;  // G of groups launched on aux_ and not yet joined
  cudaError_t launch_groups(int64_t nleaves, int G, cudaStream_t s);
  int64_t n_ = 0;
  // elements: current and scratch (x, y, z, m) + input index
  float4 *epos_ = nullptr, *tpos_ = nullptr;
  int32_t *oid_ = nullptr, *toid_ = nullptr, *idx_ = nullptr;
  int32_t *ridx_ = nullptr;  // partition: positions of the right elements by their rank
  size_t cap_e_ = 0, cap_t_ = 0, cap_o_ = 0, cap_to_ = 0, cap_i_ = 0, cap_ri_ = 0;
  DNode *nodes_ = nullptr;
  size_t cap_nodes_ = 0;
  float *ppm_ = nullptr;
  size_t cap_ppm_ = 0;
  // per-level work
  int32_t *chunk_node_ = nullptr;
  int64_t *chunk_base_ = nullptr;
  size_t cap_cn_ = 0, cap_cb_ = 0;
  double *part_ = nullptr;   // per-chunk partial sums
  size_t cap_part_ = 0;
  int32_t *left_cnt_ = nullptr;
  int64_t *left_base_ = nullptr;
  int32_t *wpre_ = nullptr;  // per chunk: each warp's left elements before its share
  int4 *chains_ = nullptr;    // the level's long swap chains (16 bytes each)
  size_t cap_lc_ = 0, cap_lb_ = 0, cap_wp_ = 0, cap_ch_ = 0;
  int64_t *scan_tmp_ = nullptr;
  size_t cap_scan_ = 0;
  int64_t *node_tmp_ = nullptr;
  size_t cap_nt_ = 0;
  int32_t *fallback_ = nullptr;
  size_t cap_fb_ = 0;
  double *tight_chunks_ = nullptr, *tight_nodes_ = nullptr;  // tight c.m. certification
  size_t cap_tc_ = 0, cap_tn_ = 0;
  int64_t *counters_ = nullptr;  // device scalars
  int64_t *h_counters_ = nullptr;  // pinned mirror
  // lists
  int32_t *leaf_ids_ = nullptr;
  size_t cap_leaf_ = 0;
  int64_t *leaf_tmp_ = nullptr;
  size_t cap_lt_ = 0;
  LeafDesc *leafdesc_ = nullptr;
  size_t cap_ld_ = 0;
  SegDesc *segs_ = nullptr;
  size_t cap_seg_ = 0;
  bool node_attr_ = false;         // k_part_node's shared-memory limit raised
  SegDesc *segs_local_ = nullptr;  // the one-pass walk's per-leaf regions
  size_t cap_segl_ = 0;
  int32_t *idx_list_ = nullptr;
  size_t cap_idx_ = 0;
  float4 *table_ = nullptr;
  size_t cap_tab_ = 0;
  PairItem *items_ = nullptr, *items_tmp_ = nullptr;
  size_t cap_items_ = 0, cap_items_tmp_ = 0;
  int32_t *gidx_ = nullptr;
  size_t cap_gidx_ = 0;
  int32_t *walk_err_ = nullptr;
  // whole subtrees in one block (k_subtree): node scratch, per-root depth
  // bookkeeping, placement offsets, per-depth totals (and their pinned copy)
  DNode *sub_nodes_ = nullptr;
  unsigned char *sub_stats_ = nullptr;  // reduced statistics of a level's nodes
  size_t cap_ss_ = 0;
  int32_t *sub_first_ = nullptr;
  int64_t *sub_hist_ = nullptr, *sub_pos_ = nullptr, *sub_tot_ = nullptr;
  size_t cap_sub_ = 0, cap_sf_ = 0, cap_sh_ = 0, cap_sp_ = 0, cap_st_ = 0;
  int64_t *h_sub_ = nullptr;
  bool sub_attr_ = false;
  bool sub_off_ = false;  // when set, every level runs in the level loop
};

// The three velocity components into tree order (out: 3 n floats).
cudaError_t launch_gather3_f32(const float *a, const float *b, const float *c, const int32_t *perm,
                               float *out, int64_t n, cudaStream_t s);
// The permuted outputs besides the velocities: x, y, z and mass from the
// tree-ordered table, phi, id and mask through perm.
cudaError_t launch_outputs(const float4 *table, const float *phi, const int64_t *id,
                           const uint16_t *mask, const int32_t *perm, float *x, float *y, float *z,
                           float *m, float *ophi, int64_t *oid, uint16_t *omask, int64_t n,
                           cudaStream_t s);
// out[i] = in[perm[i]] (into tree order).
cudaError_t launch_gather_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                              cudaStream_t s);
// pos4[i] = (x[i], y[i], z[i], m[i]).
cudaError_t launch_pack4(const float *x, const float *y, const float *z, const float *m,
                         float4 *out, int64_t n, cudaStream_t s);
// out[perm[i]] = in[i] (back to the caller's order).
cudaError_t launch_scatter_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                               cudaStream_t s);
// out[perm[i]] += in[i].
cudaError_t launch_scatter_add_f32(const float *in, const int32_t *perm, float *out, int64_t n,
                                   cudaStream_t s);
// Monopole pseudo-particle gradients passed to the particles through the
// nodes' centres of mass: xbar_k += m_k sum_{nodes P containing k} xbar_P / M_P,
// where xbar_P sits at slot n + P of the 3 arrays and M_P is the pseudo mass.
// *err (zeroed by the caller) is set on an inconsistent tree.
cudaError_t launch_pseudo_adjoint(const DNode *nodes, const std::vector<int32_t> &levels,
                                  const float4 *table, int64_t n, float *xbx, float *xby,
                                  float *xbz, int32_t *err, cudaStream_t s);
// The same for 12-point pseudo-particles: the points' position cotangents
// (slots n + 12 P + a of xbx/xby/xbz) and mass cotangents (mb, same slots)
// passed to the particles through every node's sources, centre of mass and
// tdr, top down.  xcbar (3 per node) and tdrbar (1 per node) are scratch;
// nd and ppc as the tree was built with.
cudaError_t launch_pseudo_adjoint_quad(const DNode *nodes, const std::vector<int32_t> &levels,
                                       const float4 *table, int64_t n, int32_t nd, float ppc,
                                       float *xbx, float *xby, float *xbz, float *mb, float *xcbar,
                                       float *tdrbar, int32_t *err, cudaStream_t s);

// Exclusive prefix sum of n int64 values (in may equal out); *total (device,
// may be null) receives the sum.  tmp needs scan_tmp_size(n) elements.
int64_t scan_tmp_size(int64_t n);
cudaError_t exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, int64_t *total,
                               int64_t *tmp, cudaStream_t s);

}  // namespace hsr
