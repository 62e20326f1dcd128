// rcb_host.hpp -- host side of the RCB force tree: tree build and per-leaf
// interaction lists, producing the device work description.
//
// The tree and the lists reproduce the reference exactly (same partition
// permutation, same centres of mass, same opening decisions), so the set of
// (leaf particle, list entry) pairs the GPU evaluates is the reference's:
//   build  : src/halo_finder/RCBForceTree.cxx:623-918, src/halo_finder/BGQCM.c:181-212
//   lists  : src/halo_finder/RCBForceTree.cxx:923-1197
// The build works on a packed (x, y, z, m, index) array and applies the
// resulting permutation to the caller's ten arrays once at the end, instead of
// swapping all ten arrays at every level as the reference does.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace hsr {

// Fixed pool of worker threads; parallel_for runs fn over [0, n) with dynamic
// chunks and the calling thread participating.
class Pool {
 public:
  explicit Pool(int nthreads);
  ~Pool();
  int size() const { return nthreads_; }
  void parallel_for(int64_t n, int64_t grain, const std::function<void(int64_t, int64_t)> &fn);

 private:
  void worker(int id);
  int nthreads_;
  std::vector<std::thread> threads_;
  void run_chunks();
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int64_t, int64_t)> *job_ = nullptr;
  int64_t job_n_ = 0, job_grain_ = 1;
  std::atomic<int64_t> next_{0};
  int pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Tree node (the reference's TreeNode, RCBForceTree.h:131-147), with int32
// child indices and the pseudo-particles' own slot in the position table.
// Children: c[0], c[1] (left, right) in the RCB tree, c[0..7] in the RCO
// octree; 0 = none.
struct Node {
  int64_t count = 0, offset = 0;
  int32_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool leaf() const {
    for (int i = 0; i < 8; ++i)
      if (c[i] > 0) return false;
    return true;
  }
  float tdr = 0;
  float xmin[3] = {0, 0, 0}, xmax[3] = {0, 0, 0}, xc[3] = {0, 0, 0};
  float ppm[12] = {0};
};

struct Elem {  // packed particle during the build
  float x, y, z, m;
  int32_t idx;
};

struct TreeParams {
  float min[3], max[3], min_force[3], max_force[3];
  float fsrrmax;
  float tan_oa;  // tanf(open_angle), computed once on the host
  int64_t nd;
  float ppc;
  int tdpts;
  int tree;  // 0: RCB (binary, longest axis); 1: RCO (octree, all three axes)
};

// Work description of one kick: processed leaves and their list segments.
// A segment is a run of consecutive entries of the position table: a leaf's
// particles, a small node's particles, or a node's tdpts pseudo-particles
// (stored after the n particles at n + node * tdpts).
struct Seg {
  int32_t start, count;
};

struct LeafWork {
  int64_t offset, count;   // particle range (post-permutation)
  int64_t seg_begin, seg_end;
  int64_t list_len;        // entries in the list (self included)
};

class RcbHost {
 public:
  explicit RcbHost(int nthreads);

  // Builds the tree over n particles given as SoA; afterwards perm()[k] is
  // the input index of the particle that belongs at position k, and
  // elems() holds the particles in that order.
  void build(const TreeParams &p, int64_t n, const float *x, const float *y, const float *z,
             const float *m);
  // Interaction lists of every leaf inside the force box (calcInternodeForces).
  void walk();

  // Position table entries of the pseudo-particles (x, y, z, mass) for all
  // nodes, written to out[node * tdpts + k] (4 floats each).
  void pseudo_table(float *out) const;

  int64_t n() const { return n_; }
  const std::vector<Elem> &elems() const { return elems_; }
  int64_t num_nodes() const { return num_nodes_; }
  const Node &node(int64_t i) const { return flat_[i]; }
  const std::vector<LeafWork> &leaves() const { return leaves_; }
  const std::vector<Seg> &segs() const { return segs_; }
  int64_t list_entries() const { return list_entries_; }
  int64_t pairs() const { return pairs_; }
  // pairs with each leaf's count rounded up to whole warps of 32
  int64_t padded_pairs() const;
  int64_t nonempty_leaves() const;
  Pool &pool() { return pool_; }
  const TreeParams &params() const { return p_; }

 private:
  Node &N(int64_t i) { return chunks_[i >> kChunkBits][i & (kChunk - 1)]; }
  int32_t alloc_nodes(int k);
  void node_stats(Node &T);
  void leaf_pseudo(Node &T);
  void pseudo_from_children(Node &T, const int32_t *kids, int nk);
  void build_node(int32_t tl, int depth);
  void build_node_oct(int32_t tl, int depth);
  void leaf_list(int64_t tl, std::vector<Seg> &out, std::vector<int32_t> &stack) const;

  static constexpr int kChunkBits = 13;
  static constexpr int64_t kChunk = int64_t(1) << kChunkBits;

  TreeParams p_{};
  int64_t n_ = 0;
  std::vector<Elem> elems_;
  std::vector<std::unique_ptr<Node[]>> chunks_;
  std::mutex alloc_mu_;
  std::atomic<int64_t> num_alloc_{0};
  int64_t num_nodes_ = 0;
  std::vector<Node> flat_;
  int par_depth_ = 0, par_depth_oct_ = 0;
  std::vector<LeafWork> leaves_;
  std::vector<Seg> segs_;
  int64_t list_entries_ = 0, pairs_ = 0;
  Pool pool_;
};

}  // namespace hsr
