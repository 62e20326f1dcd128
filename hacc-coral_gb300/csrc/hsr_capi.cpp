// hsr_capi.cpp -- the C ABI (include/hacc_sr.h) over the host tree and the
// sm_103a kernels.
#include "hacc_sr.h"
#include "hacc_pm.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "rcb_device.cuh"
#include "subcycle.cuh"
#include "rcb_host.hpp"
#include "sr_kernels.cuh"
#include "pm.cuh"

namespace {

using clk = std::chrono::steady_clock;
double ms_since(clk::time_point t0) {
  return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
}

// Device buffer that only grows.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes + bytes / 4, 1 << 16);
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Pinned host buffer that only grows.
struct PinBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes + bytes / 4, 1 << 16);
    cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Strict upper bound on r2 combining the pair kernel's `dist2 < fsrrmax2`
// (RCBForceTree.cxx:612-613) with the law's own `r2 <= r2max`
// (ForceLaw.cxx:140, 189), r2max = rmax^2 with FGrid's rmax (ForceLaw.cxx:32).
float cut2(int law, float fsrrmax) {
  const float fs2 = fsrrmax * fsrrmax;
  if (law == HSR_LAW_POLY5_STEP16) return fs2;
  const float rmax = 3.116326355f;
  const float r2max = rmax * rmax;
  return std::min(fs2, std::nextafter(r2max, std::numeric_limits<float>::infinity()));
}

// Squared distance bound of the batched kernel's box test: entries farther
// than this from a group's bounding box are skipped.  It sits 1e-4 (relative)
// above the pair cutoff, far beyond the few-ulp error of an FP32 r2, so every
// skipped pair would have failed the pair mask anyway.
float cull2(float rc2) { return rc2 * 1.0001f + 1e-6f; }

// Longest list range one batched item covers; longer lists are split over
// several items that add into the velocities with atomics.
constexpr int64_t kJSplit = 8192;

// Host threads that prepare the boxes of a multi-box kick concurrently.
constexpr int kBatchThreads = 4;

}  // namespace

// One background thread that issues host<->device copies of pageable arrays
// (a pageable copy holds the calling thread while it is staged), so they run
// while the calling thread drives the tree build.
class CopyWorker {
 public:
  CopyWorker() : th_([this] { loop(); }) {}
  ~CopyWorker() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    th_.join();
  }
  void submit(std::function<cudaError_t()> f) {
    {
      std::lock_guard<std::mutex> g(mu_);
      q_.push_back(std::move(f));
      ++pending_;
    }
    cv_.notify_all();
  }
  // Waits for every submitted task; returns the first error among them.
  cudaError_t wait() {
    std::unique_lock<std::mutex> g(mu_);
    done_.wait(g, [this] { return pending_ == 0; });
    const cudaError_t e = err_;
    err_ = cudaSuccess;
    return e;
  }

 private:
  void loop() {
    for (;;) {
      std::function<cudaError_t()> f;
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [this] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        f = std::move(q_.front());
        q_.pop_front();
      }
      const cudaError_t e = f();
      {
        std::lock_guard<std::mutex> g(mu_);
        if (e != cudaSuccess && err_ == cudaSuccess) err_ = e;
        --pending_;
      }
      done_.notify_all();
    }
  }
  std::mutex mu_;
  std::condition_variable cv_, done_;
  std::deque<std::function<cudaError_t()>> q_;
  int pending_ = 0;
  bool stop_ = false;
  cudaError_t err_ = cudaSuccess;
  std::thread th_;
};

// Device state of one box of a multi-box kick.
struct BoxState {
  hsr::DeviceTree tree;
  DevBuf in, out, pos4, vel, adj;
  int64_t n = 0;
  bool plain = false;
  // the box's kick parameters (a multi-box forward's tape, for its adjoint)
  int law = 0, tdpts = 1;
  int32_t nd = 0;
  float fcoeff = 0, rsm2 = 0, rc2 = 0, rcull2 = 0, ppc = 0;
  // the box's own stream: boxes of a batch are prepared concurrently
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  hsr_status status = HSR_OK;
  std::string err;
  ~BoxState() {
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }
};

// Device work of the last kick: what a pair-kernel launch reads.
struct Work {
  const float4 *table = nullptr;
  const hsr::LeafDesc *leaves = nullptr;
  const int32_t *idx = nullptr;
  const hsr::PairItem *items = nullptr;
  const int32_t *gidx = nullptr;
  float *vel = nullptr;  // 3 x n
  int64_t n = 0, nleaves = 0, nitems = 0;
  int law = 0;
  int kernel = HSR_KERNEL_BATCHED;
  int leaf_threads = 128;  // plain kernel: threads per leaf
  int group = 32;          // batched kernel: particles per group of the items
  float fcoeff = 0, rsm2 = 0, rc2 = 0, rcull2 = 0;
  bool device_built = false;
};

struct hsr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  // overlapped copies of the arrays off the critical path
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_perm = nullptr;
  std::unique_ptr<CopyWorker> copier;
  std::unique_ptr<hsr::RcbHost> host;
  hsr::DeviceTree tree;
  // host-build path
  DevBuf d_pos, d_vel, d_leaves, d_segs, d_idx, d_items, d_gidx;
  PinBuf h_pos, h_vel, h_leaves, h_segs, h_items, h_gidx;
  // device-build path: staged inputs and outputs of the ten arrays
  DevBuf d_in, d_out, d_pos4;
  // misc
  DevBuf d_law, d_flush, d_probe, d_queue, d_adj, d_res, d_sort;
  bool tape = false;  // the last call was hsr_force_fwd
  hsr_stats stats{};
  std::string err = "no error";
  bool have_lists = false;
  int last_tdpts = 1;
  int32_t tape_nd = 0;   // the taped forward's leaf size and pseudo-particle contraction
  float tape_ppc = 0.f;
  Work work;
  int batched_ctas = 0;
  // multi-box kicks
  std::vector<std::unique_ptr<BoxState>> boxes;
  DevBuf d_box_desc, d_box_items;
  bool last_was_batch = false;
  int32_t tape_boxes = 0;     // boxes whose trees are the last multi-box forward's tape
  cudaGraphExec_t batch_exec = nullptr;  // the multi-box forward's launch, replayed per call
  DevBuf d_vjp_desc;
  int32_t batch_n = 0;        // boxes of the last multi-box kick (replays)
  int64_t batch_items = 0;
  int batch_law = 0;
  int batch_group = 32;
  // launch shapes (hsr_set_tune / hsr_autotune)
  hsr_tune tune{HSR_KERNEL_BATCHED, 128, 32, 0};
  // long-range PM kick (hacc_pm.h)
  std::unique_ptr<hsr_pm::Solver> pm;
  DevBuf d_pm;
  hsr_pm_stats pm_stats{};

  // Launches a pair kernel on the current work (the batched kernel's queue
  // counter and evaluated-pair counter are reset first).
  cudaError_t launch_pairs(int kernel) {
    const Work &w = work;
    float *dv = w.vel;
    const int64_t n = w.n;
    if (kernel == HSR_KERNEL_PLAIN)
      return hsr::launch_leaf_plain(w.law, w.leaf_threads, w.table, w.leaves, w.nleaves, w.idx, dv, dv + n,
                                    dv + 2 * n, w.fcoeff, w.rsm2, w.rc2, stream);
    if (batched_ctas == 0) batched_ctas = hsr::batched_resident_ctas(device);
    cudaError_t e = d_queue.ensure(64);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d_queue.p, 0, 2 * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    return hsr::launch_pairs_batched(w.law, w.group, w.table, w.items, w.nitems, w.gidx, w.idx, dv, dv + n,
                                     dv + 2 * n, w.fcoeff, w.rsm2, w.rc2, w.rcull2,
                                     d_queue.as<unsigned long long>(), batched_ctas, stream);
  }

  // The last multi-box kick's one persistent launch, on its resident work.
  cudaError_t launch_batch_pairs() {
    cudaError_t e = cudaMemsetAsync(d_queue.p, 0, 2 * sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    return hsr::launch_pairs_batched_multi(batch_law, batch_group, d_box_desc.as<hsr::BoxDesc>(),
                                           d_box_items.as<hsr::PairItem>(), batch_items,
                                           d_queue.as<unsigned long long>(), batched_ctas, stream);
  }

  hsr_status fail(hsr_status s, const std::string &msg) {
    err = msg;
    return s;
  }
  hsr_status cuda_fail(cudaError_t e, const char *what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return HSR_ERR_CUDA;
  }
};

#define CU(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ctx->cuda_fail(e_, what); \
  } while (0)

extern "C" {

const char *hsr_version(void) { return "hacc-sr-gb300 0.1 (sm_103a)"; }

const char *hsr_last_error(const hsr_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

hsr_status hsr_create(hsr_ctx **out, int device) {
  if (!out) return HSR_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return HSR_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return HSR_ERR_ARG;
  auto *ctx = new (std::nothrow) hsr_ctx();
  if (!ctx) return HSR_ERR_NOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev2);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev3);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_perm, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete ctx;
    return HSR_ERR_CUDA;
  }
  int nth = int(std::thread::hardware_concurrency());
  ctx->host.reset(new hsr::RcbHost(std::max(1, nth)));
  *out = ctx;
  return HSR_OK;
}

hsr_status hsr_destroy(hsr_ctx *ctx) {
  if (!ctx) return HSR_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DevBuf *b : {&ctx->d_pos, &ctx->d_vel, &ctx->d_leaves, &ctx->d_segs, &ctx->d_idx, &ctx->d_law,
                    &ctx->d_flush, &ctx->d_probe, &ctx->d_items, &ctx->d_gidx, &ctx->d_queue,
                    &ctx->d_in, &ctx->d_out, &ctx->d_pos4, &ctx->d_adj, &ctx->d_box_desc,
                    &ctx->d_box_items, &ctx->d_res, &ctx->d_sort})
    b->release();
  for (PinBuf *b : {&ctx->h_pos, &ctx->h_vel, &ctx->h_leaves, &ctx->h_segs, &ctx->h_items, &ctx->h_gidx})
    b->release();
  for (auto &b : ctx->boxes)
    for (DevBuf *d : {&b->in, &b->out, &b->pos4, &b->vel, &b->adj}) d->release();
  ctx->boxes.clear();
  ctx->d_vjp_desc.release();
  if (ctx->batch_exec) cudaGraphExecDestroy(ctx->batch_exec);
  ctx->copier.reset();
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  for (cudaEvent_t ev : {ctx->ev0, ctx->ev1, ctx->ev2, ctx->ev3, ctx->ev_in, ctx->ev_perm})
    if (ev) cudaEventDestroy(ev);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  delete ctx;
  return HSR_OK;
}

hsr_status hsr_get_stats(const hsr_ctx *ctx, hsr_stats *st) {
  if (!ctx || !st) return HSR_ERR_ARG;
  *st = ctx->stats;
  return HSR_OK;
}

}  // extern "C"

namespace {

hsr_status check_params(const hsr_params *p, int64_t n, const void *const *arrs, std::string &err) {
  if (!p) return err = "null params", HSR_ERR_ARG;
  if (n < 0) return err = "negative particle count", HSR_ERR_ARG;
  if (n > 0)
    for (int i = 0; i < 10; ++i)
      if (!arrs[i]) return err = "null particle array", HSR_ERR_ARG;
  if (p->tdpts != 1 && p->tdpts != 12) return err = "tdpts must be 1 or 12", HSR_ERR_ARG;
  if (p->nd < 1) return err = "nd must be >= 1", HSR_ERR_ARG;
  if (p->law != HSR_LAW_POLY6 && p->law != HSR_LAW_POLY5_STEP16)
    return err = "unknown force law", HSR_ERR_ARG;
  if (p->kernel != HSR_KERNEL_AUTO && p->kernel != HSR_KERNEL_PLAIN && p->kernel != HSR_KERNEL_BATCHED)
    return err = "unknown kernel", HSR_ERR_ARG;
  if (p->tree != HSR_TREE_RCB && p->tree != HSR_TREE_RCO) return err = "unknown tree kind", HSR_ERR_ARG;
  // int32 position-table indices: particles plus pseudo-particles of <= 2n+1 nodes
  if (n > (int64_t(INT32_MAX) - 64) / (1 + 2 * int64_t(p->tdpts)))
    return err = "too many particles for one call", HSR_ERR_ARG;
  return HSR_OK;
}

hsr::TreeParams tree_params(const hsr_params *p) {
  hsr::TreeParams tp{};
  for (int i = 0; i < 3; ++i) {
    tp.min[i] = p->min[i];
    tp.max[i] = p->max[i];
    tp.min_force[i] = p->min_force[i];
    tp.max_force[i] = p->max_force[i];
  }
  tp.fsrrmax = p->fsrrmax;
  tp.tan_oa = std::tan(p->open_angle);
  tp.nd = p->nd;
  tp.ppc = p->ppc;
  tp.tdpts = p->tdpts;
  tp.tree = p->tree;
  return tp;
}

// Sizes of the work description produced by host_build.
struct PlanSizes {
  int64_t ntab, nleaves, nsegs, nidx;
};

// Tree build and lists on the host; fills the statistics.
PlanSizes host_build(hsr::RcbHost &H, const hsr_params *p, int64_t n, const float *x,
                     const float *y, const float *z, const float *mass, hsr_stats &st) {
  auto t0 = clk::now();
  H.build(tree_params(p), n, x, y, z, mass);
  st.t_build_ms = ms_since(t0);
  t0 = clk::now();
  H.walk();
  st.t_walk_ms = ms_since(t0);
  st.n = n;
  st.nodes = H.num_nodes();
  st.leaves = H.nonempty_leaves();
  st.processed_leaves = int64_t(H.leaves().size());
  st.list_entries = H.list_entries();
  st.pairs = H.pairs();
  return PlanSizes{n + H.num_nodes() * p->tdpts, int64_t(H.leaves().size()),
                   int64_t(H.segs().size()), H.list_entries()};
}

// Applies the tree's permutation to the caller's arrays (the reference
// permutes all ten in place) and fills the position table (particles, then
// pseudo-particles), the permuted velocities (3 x n, may be null; the
// caller's velocities are then left for the caller to overwrite) and the
// leaf/segment descriptors (may be null).
void host_fill(hsr::RcbHost &H, int64_t n, float *x, float *y, float *z, float *vx, float *vy,
               float *vz, float *mass, float *phi, int64_t *id, uint16_t *mask, float *tab,
               float *vel, hsr::LeafDesc *ld, hsr::SegDesc *sd,
               std::vector<int64_t> *list_begin = nullptr) {
  const auto &el = H.elems();
  hsr::Pool &pool = H.pool();
  pool.parallel_for(n, 1 << 15, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const hsr::Elem &q = el[i];
      float *o = tab + 4 * i;
      o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.m;
      if (vel) {
        vel[i] = vx[q.idx];
        vel[n + i] = vy[q.idx];
        vel[2 * n + i] = vz[q.idx];
      }
    }
  });
  std::vector<float> tf(static_cast<size_t>(n));
  auto gather_f = [&](float *a) {
    pool.parallel_for(n, 1 << 15, [&](int64_t b, int64_t e) {
      for (int64_t i = b; i < e; ++i) tf[i] = a[el[i].idx];
    });
    std::memcpy(a, tf.data(), size_t(n) * 4);
  };
  gather_f(phi);
  if (!vel) {
    gather_f(vx);
    gather_f(vy);
    gather_f(vz);
  }
  {
    std::vector<int64_t> ti(static_cast<size_t>(n));
    std::vector<uint16_t> tm(static_cast<size_t>(n));
    pool.parallel_for(n, 1 << 15, [&](int64_t b, int64_t e) {
      for (int64_t i = b; i < e; ++i) {
        ti[i] = id[el[i].idx];
        tm[i] = mask[el[i].idx];
      }
    });
    if (n) {
      std::memcpy(id, ti.data(), size_t(n) * 8);
      std::memcpy(mask, tm.data(), size_t(n) * 2);
    }
  }
  pool.parallel_for(n, 1 << 15, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      x[i] = el[i].x;
      y[i] = el[i].y;
      z[i] = el[i].z;
      mass[i] = el[i].m;
    }
  });
  H.pseudo_table(tab + 4 * n);
  if (!ld) return;
  const auto &leaves = H.leaves();
  const auto &segs = H.segs();
  const int64_t nl = int64_t(leaves.size());
  std::vector<int64_t> lb(static_cast<size_t>(nl));
  int64_t run = 0;
  for (int64_t l = 0; l < nl; ++l) {
    lb[l] = run;
    run += leaves[l].list_len;
  }
  if (list_begin) *list_begin = lb;
  pool.parallel_for(nl, 64, [&](int64_t b, int64_t e) {
    for (int64_t l = b; l < e; ++l) {
      const auto &L = leaves[l];
      hsr::LeafDesc d{};
      d.offset = int32_t(L.offset);
      d.count = int32_t(L.count);
      d.list_len = int32_t(L.list_len);
      d.kept_len = d.list_len;  // host lists are not pruned
      d.list_begin = lb[l];
      ld[l] = d;
      int64_t dst = lb[l];
      for (int64_t s = L.seg_begin; s < L.seg_end; ++s) {
        sd[s] = hsr::SegDesc{segs[s].start, segs[s].count, dst};
        dst += segs[s].count;
      }
    }
  });
}

// Expands the segments of the lists into entries (x, y, z, m) and/or
// position-table indices.
void export_lists(const hsr::RcbHost &H, const float *tab, int64_t *leaf_offset,
                  int64_t *leaf_count, int64_t *list_ptr, float *ex, float *ey, float *ez,
                  float *em, int64_t *eidx) {
  int64_t run = 0;
  for (size_t l = 0; l < H.leaves().size(); ++l) {
    const auto &L = H.leaves()[l];
    if (leaf_offset) leaf_offset[l] = L.offset;
    if (leaf_count) leaf_count[l] = L.count;
    if (list_ptr) list_ptr[l] = run;
    for (int64_t s = L.seg_begin; s < L.seg_end; ++s) {
      const auto &sg = H.segs()[s];
      for (int32_t q = 0; q < sg.count; ++q) {
        const int64_t t = int64_t(sg.start) + q;
        if (ex) {
          const float *e = tab + 4 * t;
          ex[run] = e[0];
          ey[run] = e[1];
          ez[run] = e[2];
          em[run] = e[3];
        }
        if (eidx) eidx[run] = t;
        ++run;
      }
    }
  }
  if (list_ptr) list_ptr[H.leaves().size()] = run;
}

// Splits each processed leaf into ceil(count/32) spatially compact groups
// (recursive halving along the longest axis, left part a multiple of 32) and
// emits one batched-kernel item per group and list chunk of at most `jsplit`
// entries, sorted by list length, longest first.  gidx has n entries: each
// leaf's range holds a permutation of its particles, grouped.
void make_items(hsr::RcbHost &H, const std::vector<int64_t> &list_begin, int64_t jsplit, int G,
                std::vector<int32_t> &gidx, std::vector<hsr::PairItem> &items) {
  const auto &leaves = H.leaves();
  const auto &el = H.elems();
  const int64_t nl = int64_t(leaves.size());
  gidx.resize(size_t(H.n()));
  std::vector<int64_t> item_base(size_t(nl) + 1, 0);
  for (int64_t l = 0; l < nl; ++l) {
    const int64_t ng = std::max<int64_t>(0, (leaves[l].count + G - 1) / G);
    const int64_t nch = std::max<int64_t>(1, (leaves[l].list_len + jsplit - 1) / jsplit);
    item_base[l + 1] = item_base[l] + ng * nch;
  }
  items.resize(size_t(item_base[nl]));
  H.pool().parallel_for(nl, 16, [&](int64_t b, int64_t e) {
    std::vector<int32_t> tmp;
    std::vector<std::pair<int32_t, int32_t>> stack, out;
    for (int64_t l = b; l < e; ++l) {
      const auto &L = leaves[l];
      if (L.count <= 0) continue;  // an empty root leaf has no groups and no items
      tmp.resize(size_t(L.count));
      for (int64_t i = 0; i < L.count; ++i) tmp[i] = int32_t(L.offset + i);
      out.clear();
      stack.assign(1, {0, int32_t(L.count)});
      while (!stack.empty()) {
        auto [a, c] = stack.back();
        stack.pop_back();
        if (c <= G) {
          if (c > 0) out.push_back({a, c});
          continue;
        }
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (int32_t i = a; i < a + c; ++i) {
          const hsr::Elem &q = el[tmp[i]];
          const float v[3] = {q.x, q.y, q.z};
          for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], v[d]);
            hi[d] = std::max(hi[d], v[d]);
          }
        }
        int d = 0;
        for (int k = 1; k < 3; ++k)
          if (hi[k] - lo[k] > hi[d] - lo[d]) d = k;
        const int32_t ng = (c + G - 1) / G;
        const int32_t left = G * ((ng + 1) / 2);
        auto key = [&](int32_t i) {
          const hsr::Elem &q = el[i];
          return d == 0 ? q.x : d == 1 ? q.y : q.z;
        };
        std::nth_element(tmp.begin() + a, tmp.begin() + a + left, tmp.begin() + a + c,
                         [&](int32_t u, int32_t v) { return key(u) < key(v); });
        stack.push_back({a + left, c - left});
        stack.push_back({a, left});
      }
      std::copy(tmp.begin(), tmp.end(), gidx.begin() + L.offset);
      const int64_t nch = std::max<int64_t>(1, (L.list_len + jsplit - 1) / jsplit);
      int64_t k = item_base[l];
      for (const auto &g : out)
        for (int64_t c = 0; c < nch; ++c) {
          hsr::PairItem it{};
          it.j_begin = list_begin[l] + c * jsplit;
          it.j_len = int32_t(std::min<int64_t>(jsplit, L.list_len - c * jsplit));
          it.g_begin = int32_t(L.offset + g.first);
          it.g_count = g.second;
          it.flags = nch > 1 ? 1 : 0;
          items[k++] = it;
        }
    }
  });
  std::stable_sort(items.begin(), items.end(), [](const hsr::PairItem &a, const hsr::PairItem &b) {
    return a.j_len > b.j_len;
  });
}

}  // namespace

struct hsr_lists {
  std::unique_ptr<hsr::RcbHost> host;
  std::vector<float> tab;
  hsr_stats st{};
};

namespace {

void set_work_params(Work &w, const hsr_params *p, int64_t n, const hsr_tune &t) {
  w.n = n;
  w.law = p->law;
  w.fcoeff = p->fcoeff;
  w.rsm2 = p->rsm * p->rsm;
  w.rc2 = cut2(p->law, p->fsrrmax);
  w.rcull2 = cull2(w.rc2);
  w.kernel = p->kernel == HSR_KERNEL_AUTO ? t.kernel : p->kernel;
  w.leaf_threads = t.leaf_threads;
  w.group = t.group;
}

// Tree and lists on the host (rcb_host.cpp), pair kernel on the device.
hsr_status kick_host_build(hsr_ctx *ctx, const hsr_params *p, int64_t n, float *x, float *y,
                           float *z, float *vx, float *vy, float *vz, float *mass, float *phi,
                           int64_t *id, uint16_t *mask, hsr_stats &st) {
  hsr::RcbHost &H = *ctx->host;
  const PlanSizes ps = host_build(H, p, n, x, y, z, mass, st);
  CU(ctx->h_pos.ensure(size_t(std::max<int64_t>(ps.ntab, 1)) * 16), "cudaHostAlloc(pos)");
  CU(ctx->h_vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4), "cudaHostAlloc(vel)");
  CU(ctx->h_leaves.ensure(size_t(std::max<int64_t>(ps.nleaves, 1)) * sizeof(hsr::LeafDesc)),
     "cudaHostAlloc(leaves)");
  CU(ctx->h_segs.ensure(size_t(std::max<int64_t>(ps.nsegs, 1)) * sizeof(hsr::SegDesc)),
     "cudaHostAlloc(segs)");
  float *hp = ctx->h_pos.as<float>();
  float *hv = ctx->h_vel.as<float>();
  auto *hl = ctx->h_leaves.as<hsr::LeafDesc>();
  auto *hs = ctx->h_segs.as<hsr::SegDesc>();
  std::vector<int64_t> list_begin;
  host_fill(H, n, x, y, z, vx, vy, vz, mass, phi, id, mask, hp, hv, hl, hs, &list_begin);
  Work &w = ctx->work;
  set_work_params(w, p, n, ctx->tune);
  const bool plain = w.kernel == HSR_KERNEL_PLAIN;
  int64_t nitems = 0;
  if (!plain) {
    std::vector<int32_t> gidx;
    std::vector<hsr::PairItem> items;
    make_items(H, list_begin, kJSplit, w.group, gidx, items);
    nitems = int64_t(items.size());
    CU(ctx->h_items.ensure(std::max<size_t>(items.size(), 1) * sizeof(hsr::PairItem)), "cudaHostAlloc(items)");
    CU(ctx->h_gidx.ensure(std::max<size_t>(gidx.size(), 1) * 4), "cudaHostAlloc(gidx)");
    std::memcpy(ctx->h_items.p, items.data(), items.size() * sizeof(hsr::PairItem));
    std::memcpy(ctx->h_gidx.p, gidx.data(), gidx.size() * 4);
  }
  cudaStream_t s = ctx->stream;
  CU(ctx->d_pos.ensure(size_t(std::max<int64_t>(ps.ntab, 1)) * 16), "cudaMalloc(pos)");
  CU(ctx->d_vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4), "cudaMalloc(vel)");
  CU(ctx->d_leaves.ensure(size_t(std::max<int64_t>(ps.nleaves, 1)) * sizeof(hsr::LeafDesc)),
     "cudaMalloc(leaves)");
  CU(ctx->d_segs.ensure(size_t(std::max<int64_t>(ps.nsegs, 1)) * sizeof(hsr::SegDesc)),
     "cudaMalloc(segs)");
  CU(ctx->d_idx.ensure(size_t(std::max<int64_t>(ps.nidx, 1)) * 4), "cudaMalloc(idx)");
  CU(cudaMemcpyAsync(ctx->d_pos.p, hp, size_t(ps.ntab) * 16, cudaMemcpyHostToDevice, s), "H2D pos");
  CU(cudaMemcpyAsync(ctx->d_vel.p, hv, size_t(3 * n) * 4, cudaMemcpyHostToDevice, s), "H2D vel");
  CU(cudaMemcpyAsync(ctx->d_leaves.p, hl, size_t(ps.nleaves) * sizeof(hsr::LeafDesc),
                     cudaMemcpyHostToDevice, s), "H2D leaves");
  CU(cudaMemcpyAsync(ctx->d_segs.p, hs, size_t(ps.nsegs) * sizeof(hsr::SegDesc),
                     cudaMemcpyHostToDevice, s), "H2D segs");
  int64_t h2d_items = 0;
  if (!plain) {
    CU(ctx->d_items.ensure(size_t(std::max<int64_t>(nitems, 1)) * sizeof(hsr::PairItem)), "cudaMalloc(items)");
    CU(ctx->d_gidx.ensure(size_t(std::max<int64_t>(n, 1)) * 4), "cudaMalloc(gidx)");
    CU(cudaMemcpyAsync(ctx->d_items.p, ctx->h_items.p, size_t(nitems) * sizeof(hsr::PairItem),
                       cudaMemcpyHostToDevice, s), "H2D items");
    CU(cudaMemcpyAsync(ctx->d_gidx.p, ctx->h_gidx.p, size_t(n) * 4, cudaMemcpyHostToDevice, s),
       "H2D gidx");
    h2d_items = nitems * int64_t(sizeof(hsr::PairItem)) + 4 * n;
  }
  int64_t launches = 0;
  CU(hsr::launch_expand_segments(ctx->d_segs.as<hsr::SegDesc>(), ps.nsegs, ctx->d_idx.as<int32_t>(), s),
     "expand kernel");
  launches += ps.nsegs > 0;
  w.table = ctx->d_pos.as<float4>();
  w.leaves = ctx->d_leaves.as<hsr::LeafDesc>();
  w.idx = ctx->d_idx.as<int32_t>();
  w.items = ctx->d_items.as<hsr::PairItem>();
  w.gidx = ctx->d_gidx.as<int32_t>();
  w.vel = ctx->d_vel.as<float>();
  w.nleaves = ps.nleaves;
  w.nitems = nitems;
  w.device_built = false;
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(ctx->launch_pairs(w.kernel), "pair kernel");
  launches += plain ? ps.nleaves > 0 : nitems > 0;
  CU(cudaEventRecord(ctx->ev1, s), "event");
  float *dv = w.vel;
  CU(cudaMemcpyAsync(hv, dv, size_t(3 * n) * 4, cudaMemcpyDeviceToHost, s), "D2H vel");
  unsigned long long counters[2] = {0, 0};
  if (!plain) CU(cudaMemcpyAsync(counters, ctx->d_queue.p, sizeof(counters), cudaMemcpyDeviceToHost, s),
                 "D2H counters");
  CU(cudaStreamSynchronize(s), "kernel execution");
  st.evaluated_pairs = plain ? H.padded_pairs() : int64_t(counters[1]);
  float fms = 0;
  CU(cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1), "event time");
  st.t_force_ms = fms;
  H.pool().parallel_for(n, 1 << 15, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      vx[i] = hv[i];
      vy[i] = hv[n + i];
      vz[i] = hv[2 * n + i];
    }
  });
  st.kernel_launches = launches;
  st.work_items = nitems;
  st.h2d_bytes = ps.ntab * 16 + 3 * n * 4 + ps.nleaves * int64_t(sizeof(hsr::LeafDesc)) +
                 ps.nsegs * int64_t(sizeof(hsr::SegDesc)) + h2d_items;
  st.d2h_bytes = 3 * n * 4 + (plain ? 0 : 16);
  return HSR_OK;
}

// Offsets of the ten arrays inside one staging region (8 float arrays, the
// int64 ids, the uint16 masks), each 256-byte aligned.
struct ArrayLayout {
  size_t f[8], id, mask, bytes;
  explicit ArrayLayout(int64_t n) {
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t o = 0;
    for (int i = 0; i < 8; ++i) {
      f[i] = o;
      o = up(o + size_t(n) * 4);
    }
    id = o;
    o = up(o + size_t(n) * 8);
    mask = o;
    o = up(o + size_t(n) * 2);
    bytes = std::max<size_t>(o, 256);
  }
};

// Tree, lists, work items and the kick all on the device (rcb_device.cu).
hsr_status kick_device_build(hsr_ctx *ctx, const hsr_params *p, int64_t n, float *x, float *y,
                             float *z, float *vx, float *vy, float *vz, float *mass, float *phi,
                             int64_t *id, uint16_t *mask, int32_t mem, hsr_stats &st) {
  cudaStream_t s = ctx->stream;
  const ArrayLayout A(n);
  float *arr[8] = {x, y, z, vx, vy, vz, mass, phi};
  CU(ctx->d_out.ensure(A.bytes), "cudaMalloc(out)");
  CU(ctx->d_pos4.ensure(size_t(std::max<int64_t>(n, 1)) * 16), "cudaMalloc(pos4)");
  const float *in[8];
  const int64_t *in_id;
  const uint16_t *in_mask;
  char *ob = ctx->d_out.as<char>();
  const auto t_in = clk::now();
  // Host arrays: x, y, z and mass (the tree build's input) are copied on the
  // critical path; the other six arrays are copied by the context's copy
  // thread on its own stream while the tree is built, and the permuted x, y,
  // z, mass, phi, id and mask go back while the lists and the kick run.
  const bool overlap = mem == HSR_MEM_HOST && n > 0;
  // on every return, no copy of the caller's arrays may still be in flight
  struct CopyGuard {
    CopyWorker *w = nullptr;
    ~CopyGuard() {
      if (w) w->wait();
    }
  } guard;
  if (mem == HSR_MEM_HOST) {
    CU(ctx->d_in.ensure(A.bytes), "cudaMalloc(in)");
    char *ib = ctx->d_in.as<char>();
    for (int i = 0; i < 8; ++i) in[i] = reinterpret_cast<const float *>(ib + A.f[i]);
    for (int i : {0, 1, 2, 6})
      CU(cudaMemcpyAsync(ib + A.f[i], arr[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D positions");
    in_id = reinterpret_cast<const int64_t *>(ib + A.id);
    in_mask = reinterpret_cast<const uint16_t *>(ib + A.mask);
    st.h2d_bytes = n * 42;
    if (overlap) {
      if (!ctx->copier) ctx->copier.reset(new (std::nothrow) CopyWorker());
      if (!ctx->copier) return ctx->fail(HSR_ERR_NOMEM, "copy thread");
      guard.w = ctx->copier.get();
      const int dev = ctx->device;
      cudaStream_t s2 = ctx->copy_stream;
      cudaEvent_t ev = ctx->ev_in;
      float *src[4] = {arr[3], arr[4], arr[5], arr[7]};
      char *dst[4] = {ib + A.f[3], ib + A.f[4], ib + A.f[5], ib + A.f[7]};
      char *did = ib + A.id, *dmask = ib + A.mask;
      const int64_t *hid = id;
      const uint16_t *hmask = mask;
      ctx->copier->submit([=]() -> cudaError_t {
        cudaError_t e = cudaSetDevice(dev);
        for (int i = 0; i < 4 && e == cudaSuccess; ++i)
          e = cudaMemcpyAsync(dst[i], src[i], size_t(n) * 4, cudaMemcpyHostToDevice, s2);
        if (e == cudaSuccess) e = cudaMemcpyAsync(did, hid, size_t(n) * 8, cudaMemcpyHostToDevice, s2);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dmask, hmask, size_t(n) * 2, cudaMemcpyHostToDevice, s2);
        if (e == cudaSuccess) e = cudaEventRecord(ev, s2);
        return e;
      });
    }
  } else {
    for (int i = 0; i < 8; ++i) in[i] = arr[i];
    in_id = id;
    in_mask = mask;
  }
  int64_t launches = 0;
  float4 *pos4 = ctx->d_pos4.as<float4>();
  CU(cudaStreamSynchronize(s), "host to device copies");
  st.t_h2d_ms = ms_since(t_in);
  CU(hsr::launch_pack4(in[0], in[1], in[2], in[6], pos4, n, s), "pack kernel");
  ++launches;
  hsr::TreeConfig cfg{};
  for (int i = 0; i < 3; ++i) {
    cfg.min[i] = p->min[i];
    cfg.max[i] = p->max[i];
    cfg.min_force[i] = p->min_force[i];
    cfg.max_force[i] = p->max_force[i];
  }
  cfg.fsrrmax = p->fsrrmax;
  cfg.prune2 = cull2(cut2(p->law, p->fsrrmax));
  cfg.tan_oa = std::tan(p->open_angle);  // host tanf, as the reference computes it
  cfg.ppc = p->ppc;
  cfg.nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
  cfg.tdpts = p->tdpts;
  cfg.group = ctx->tune.group;
  {
    const char *f = std::getenv("HSR_FORCE_CM_FALLBACK");  // test hook
    cfg.force_cm_fallback = (f && (f[0] == '1' || f[0] == '2')) ? f[0] - '0' : 0;
  }
  CU(cudaEventRecord(ctx->ev3, s), "event");
  const auto tb = clk::now();
  cudaError_t e = ctx->tree.build(cfg, n, pos4, kJSplit, s);
  if (e != cudaSuccess) {
    if (ctx->tree.error()) return ctx->fail(HSR_ERR_UNSUPPORTED, ctx->tree.error());
    return ctx->cuda_fail(e, "device tree build");
  }
  st.t_build_ms = ctx->tree.build_ms();
  st.t_walk_ms = ctx->tree.lists_ms();
  (void)tb;
  const hsr::DeviceTreeInfo &ti = ctx->tree.info();
  launches += ti.launches;
  const int32_t *perm = ctx->tree.perm();
  if (overlap) {
    CU(ctx->copier->wait(), "H2D arrays (copy thread)");
    CU(cudaStreamWaitEvent(s, ctx->ev_in, 0), "wait for the copies");
  }
  // outputs in tree order: velocities to the kick buffer, the rest to d_out
  Work &w = ctx->work;
  set_work_params(w, p, n, ctx->tune);
  float *ovx = reinterpret_cast<float *>(ob + A.f[3]), *ovy = reinterpret_cast<float *>(ob + A.f[4]),
        *ovz = reinterpret_cast<float *>(ob + A.f[5]);
  CU(ctx->d_vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4), "cudaMalloc(vel)");
  float *dv = ctx->d_vel.as<float>();
  CU(hsr::launch_gather3_f32(in[3], in[4], in[5], perm, dv, n, s), "gather velocities");
  // the other permuted outputs ahead of the pair kernel (which takes every
  // SM), so that their copies back overlap it
  CU(hsr::launch_outputs(ctx->tree.table(), in[7], in_id, in_mask, perm,
                         reinterpret_cast<float *>(ob + A.f[0]), reinterpret_cast<float *>(ob + A.f[1]),
                         reinterpret_cast<float *>(ob + A.f[2]), reinterpret_cast<float *>(ob + A.f[6]),
                         reinterpret_cast<float *>(ob + A.f[7]), reinterpret_cast<int64_t *>(ob + A.id),
                         reinterpret_cast<uint16_t *>(ob + A.mask), n, s),
     "gather outputs");
  launches += 2;
  if (overlap) {
    // the permuted arrays other than the velocities go back now
    CU(cudaEventRecord(ctx->ev_perm, s), "event");
    CU(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_perm, 0), "wait for the outputs");
    const int dev = ctx->device;
    cudaStream_t s2 = ctx->copy_stream;
    float *dst[5] = {arr[0], arr[1], arr[2], arr[6], arr[7]};
    const char *src[5] = {ob + A.f[0], ob + A.f[1], ob + A.f[2], ob + A.f[6], ob + A.f[7]};
    const char *sid = ob + A.id, *smask = ob + A.mask;
    int64_t *hid = id;
    uint16_t *hmask = mask;
    ctx->copier->submit([=]() -> cudaError_t {
      cudaError_t e = cudaSetDevice(dev);
      for (int i = 0; i < 5 && e == cudaSuccess; ++i)
        e = cudaMemcpyAsync(dst[i], src[i], size_t(n) * 4, cudaMemcpyDeviceToHost, s2);
      if (e == cudaSuccess) e = cudaMemcpyAsync(hid, sid, size_t(n) * 8, cudaMemcpyDeviceToHost, s2);
      if (e == cudaSuccess) e = cudaMemcpyAsync(hmask, smask, size_t(n) * 2, cudaMemcpyDeviceToHost, s2);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s2);
      return e;
    });
  }
  w.table = ctx->tree.table();
  w.leaves = ctx->tree.leaves();
  w.idx = ctx->tree.index();
  w.items = ctx->tree.items();
  w.gidx = ctx->tree.gidx();
  w.group = ctx->tree.group();
  w.vel = dv;
  w.nleaves = ti.processed_leaves;
  w.nitems = ti.items;
  w.device_built = true;
  const bool plain = w.kernel == HSR_KERNEL_PLAIN;
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(ctx->launch_pairs(w.kernel), "pair kernel");
  launches += plain ? w.nleaves > 0 : w.nitems > 0;
  CU(cudaEventRecord(ctx->ev1, s), "event");
  // kicked velocities into the output slots, then everything back
  CU(cudaMemcpyAsync(ovx, dv, size_t(n) * 4, cudaMemcpyDeviceToDevice, s), "copy vx");
  CU(cudaMemcpyAsync(ovy, dv + n, size_t(n) * 4, cudaMemcpyDeviceToDevice, s), "copy vy");
  CU(cudaMemcpyAsync(ovz, dv + 2 * n, size_t(n) * 4, cudaMemcpyDeviceToDevice, s), "copy vz");
  const cudaMemcpyKind back = mem == HSR_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int i = 0; i < 8; ++i)
    if (!overlap || (i >= 3 && i <= 5))
      CU(cudaMemcpyAsync(arr[i], ob + A.f[i], size_t(n) * 4, back, s), "copy arrays back");
  if (!overlap) {
    CU(cudaMemcpyAsync(id, ob + A.id, size_t(n) * 8, back, s), "copy ids back");
    CU(cudaMemcpyAsync(mask, ob + A.mask, size_t(n) * 2, back, s), "copy masks back");
  }
  unsigned long long counters[2] = {0, 0};
  if (!plain) CU(cudaMemcpyAsync(counters, ctx->d_queue.p, sizeof(counters), cudaMemcpyDeviceToHost, s),
                 "D2H counters");
  CU(cudaEventRecord(ctx->ev2, s), "event");
  CU(cudaStreamSynchronize(s), "kernel execution");
  if (overlap) CU(ctx->copier->wait(), "D2H arrays (copy thread)");
  float fms = 0, oms = 0;
  CU(cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1), "event time");
  CU(cudaEventElapsedTime(&oms, ctx->ev1, ctx->ev2), "event time");
  st.t_force_ms = fms;
  st.t_d2h_ms = oms;
  st.n = n;
  st.nodes = ti.nodes;
  st.leaves = 0;
  st.processed_leaves = ti.processed_leaves;
  st.list_entries = ti.list_entries;
  st.pairs = ti.pairs;
  st.evaluated_pairs = plain ? ctx->tree.padded_pairs() : int64_t(counters[1]);
  st.work_items = ti.items;
  st.cm_fallbacks = ti.cm_fallbacks;
  st.kernel_launches = launches;
  if (mem == HSR_MEM_HOST) st.d2h_bytes = n * 42 + (plain ? 0 : 16);
  return HSR_OK;
}

}  // namespace

namespace {

// The sub-cycles of hsr_subcycle on arrays already resident on the device
// (f: x, y, z, vx, vy, vz, mass, phi): nsub times stream, resort, masses = 1,
// kick, stream.  Statistics of the kicks are summed into `total`.
hsr_status subcycle_resident(hsr_ctx *ctx, const hsr_subcycle_params *sp, int64_t n, float **f,
                             int64_t *ids, uint16_t *msk, int64_t *inbox, hsr_stats &total) {
  cudaStream_t s = ctx->stream;
  CU(ctx->d_sort.ensure(hsr::resort_scratch_bytes(n)), "cudaMalloc(sort)");
  // map1's prefactor in float, as the reference computes it
  const float pf = std::pow(sp->pp, float(1.0 + 1.0 / sp->alpha));
  const float prefactor = float(1.0 / (sp->alpha * sp->adot * pf));
  const float pt = prefactor * sp->tau;
  for (int32_t step = 0; step < sp->nsub; ++step) {
    if (!sp->skip_stream) CU(hsr::launch_stream(f[0], f[1], f[2], f[3], f[4], f[5], n, pt, s), "stream");
    if (!sp->skip_kick) {
      CU(hsr::resort_by_cell(n, sp->ng, f, ids, msk, ctx->d_sort.p, inbox, s), "resort");
      CU(hsr::launch_fill(f[6], n, 1.0f, s), "masses");
      hsr_stats st{};
      hsr_status r = kick_device_build(ctx, &sp->kick, *inbox, f[0], f[1], f[2], f[3], f[4], f[5],
                                       f[6], f[7], ids, msk, HSR_MEM_DEVICE, st);
      if (r != HSR_OK) return r;
      total.pairs += st.pairs;
      total.evaluated_pairs += st.evaluated_pairs;
      total.list_entries += st.list_entries;
      total.processed_leaves += st.processed_leaves;
      total.nodes += st.nodes;
      total.t_build_ms += st.t_build_ms;
      total.t_walk_ms += st.t_walk_ms;
      total.t_force_ms += st.t_force_ms;
      total.cm_fallbacks += st.cm_fallbacks;
      total.kernel_launches += st.kernel_launches;
    }
    if (!sp->skip_stream) CU(hsr::launch_stream(f[0], f[1], f[2], f[3], f[4], f[5], n, pt, s), "stream");
  }
  return HSR_OK;
}

}  // namespace

extern "C" {

hsr_status hsr_rcb_kick(hsr_ctx *ctx, const hsr_params *p, int64_t n, float *x, float *y, float *z,
                        float *vx, float *vy, float *vz, float *mass, float *phi, int64_t *id,
                        uint16_t *mask, int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t_start = clk::now();
  const void *arrs[10] = {x, y, z, vx, vy, vz, mass, phi, id, mask};
  if (hsr_status e = check_params(p, n, arrs, ctx->err)) return e;
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  if (p->build != HSR_BUILD_DEVICE && p->build != HSR_BUILD_HOST)
    return ctx->fail(HSR_ERR_ARG, "bad build location");
  // the RCO octree is built on the host
  const bool host_build = p->build == HSR_BUILD_HOST || p->tree == HSR_TREE_RCO;
  if (host_build && mem != HSR_MEM_HOST)
    return ctx->fail(HSR_ERR_UNSUPPORTED, "the host build (and the RCO tree) takes host arrays");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->have_lists = false;
  ctx->tape = false;
  ctx->last_was_batch = false;
  ctx->tape_boxes = 0;
  hsr_stats st{};
  hsr_status r = host_build
                     ? kick_host_build(ctx, p, n, x, y, z, vx, vy, vz, mass, phi, id, mask, st)
                     : kick_device_build(ctx, p, n, x, y, z, vx, vy, vz, mass, phi, id, mask, mem, st);
  if (r != HSR_OK) return r;
  st.t_total_ms = ms_since(t_start);
  ctx->stats = st;
  ctx->have_lists = true;
  ctx->last_tdpts = p->tdpts;
  return HSR_OK;
}

hsr_status hsr_lists_size(const hsr_ctx *ctx, int64_t *nleaves, int64_t *nentries) {
  if (!ctx || !nleaves || !nentries) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  *nleaves = ctx->work.device_built ? ctx->tree.info().processed_leaves
                                    : int64_t(ctx->host->leaves().size());
  *nentries = ctx->work.device_built ? ctx->tree.info().list_entries : ctx->host->list_entries();
  return HSR_OK;
}

hsr_status hsr_lists_export(const hsr_ctx *ctx_c, int64_t *leaf_offset, int64_t *leaf_count,
                            int64_t *list_ptr, float *ex, float *ey, float *ez, float *em) {
  hsr_ctx *ctx = const_cast<hsr_ctx *>(ctx_c);
  if (!ctx || !leaf_offset || !leaf_count || !list_ptr || !ex || !ey || !ez || !em) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  if (!ctx->work.device_built) {
    export_lists(*ctx->host, ctx->h_pos.as<float>(), leaf_offset, leaf_count, list_ptr, ex, ey, ez,
                 em, nullptr);
    return HSR_OK;
  }
  // device-built lists: copy the descriptors and the table, expand here
  const auto &ti = ctx->tree.info();
  const int64_t nl = ti.processed_leaves, ns = ti.segments;
  const int64_t ntab = ctx->work.n + ti.nodes * ctx->last_tdpts;
  std::vector<hsr::LeafDesc> ld(static_cast<size_t>(std::max<int64_t>(nl, 1)));
  std::vector<hsr::SegDesc> sd(static_cast<size_t>(std::max<int64_t>(ns, 1)));
  std::vector<float4> tab(static_cast<size_t>(std::max<int64_t>(ntab, 1)));
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  CU(cudaMemcpyAsync(ld.data(), ctx->tree.leaves(), size_t(nl) * sizeof(hsr::LeafDesc),
                     cudaMemcpyDeviceToHost, s), "D2H leaves");
  CU(cudaMemcpyAsync(sd.data(), ctx->tree.segs(), size_t(ns) * sizeof(hsr::SegDesc),
                     cudaMemcpyDeviceToHost, s), "D2H segments");
  CU(cudaMemcpyAsync(tab.data(), ctx->tree.table(), size_t(ntab) * sizeof(float4),
                     cudaMemcpyDeviceToHost, s), "D2H table");
  CU(cudaStreamSynchronize(s), "list export");
  // segments are stored leaf after leaf in list order
  int64_t seg = 0;
  for (int64_t l = 0; l < nl; ++l) {
    leaf_offset[l] = ld[l].offset;
    leaf_count[l] = ld[l].count;
    list_ptr[l] = ld[l].list_begin;
    int64_t run = ld[l].list_begin;
    const int64_t end = ld[l].list_begin + ld[l].list_len;
    while (run < end && seg < ns) {
      const hsr::SegDesc &g = sd[seg++];
      for (int32_t q = 0; q < g.count; ++q) {
        const float4 e = tab[size_t(g.start) + q];
        ex[run] = e.x;
        ey[run] = e.y;
        ez[run] = e.z;
        em[run] = e.w;
        ++run;
      }
    }
  }
  list_ptr[nl] = ti.list_entries;
  return HSR_OK;
}

hsr_status hsr_subcycle(hsr_ctx *ctx, const hsr_subcycle_params *sp, int64_t n, float *x,
                        float *y, float *z, float *vx, float *vy, float *vz, float *mass,
                        float *phi, int64_t *id, uint16_t *mask, int32_t mem, int64_t *n_inbox) {
  if (!ctx) return HSR_ERR_ARG;
  if (!sp) return ctx->fail(HSR_ERR_ARG, "null parameters");
  const auto t_start = clk::now();
  const void *arrs[10] = {x, y, z, vx, vy, vz, mass, phi, id, mask};
  if (hsr_status e = check_params(&sp->kick, n, arrs, ctx->err)) return e;
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  if (sp->kick.tree != HSR_TREE_RCB)
    return ctx->fail(HSR_ERR_UNSUPPORTED, "the device sub-cycle builds the RCB tree only");
  if (sp->nsub < 0 || sp->ng[0] < 1 || sp->ng[1] < 1 || sp->ng[2] < 1 ||
      double(sp->ng[0]) * sp->ng[1] * sp->ng[2] >= 4294967295.0)
    return ctx->fail(HSR_ERR_ARG, "bad sub-cycle count or grid");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->tape = false;
  ctx->last_was_batch = false;
  ctx->tape_boxes = 0;
  cudaStream_t s = ctx->stream;
  // resident arrays
  const ArrayLayout A(n);
  float *f[8] = {x, y, z, vx, vy, vz, mass, phi};
  int64_t *ids = id;
  uint16_t *msk = mask;
  if (mem == HSR_MEM_HOST) {
    CU(ctx->d_res.ensure(A.bytes), "cudaMalloc(resident)");
    char *rb = ctx->d_res.as<char>();
    for (int i = 0; i < 8; ++i) {
      CU(cudaMemcpyAsync(rb + A.f[i], f[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D arrays");
      f[i] = reinterpret_cast<float *>(rb + A.f[i]);
    }
    CU(cudaMemcpyAsync(rb + A.id, id, size_t(n) * 8, cudaMemcpyHostToDevice, s), "H2D ids");
    CU(cudaMemcpyAsync(rb + A.mask, mask, size_t(n) * 2, cudaMemcpyHostToDevice, s), "H2D masks");
    ids = reinterpret_cast<int64_t *>(rb + A.id);
    msk = reinterpret_cast<uint16_t *>(rb + A.mask);
  }
  hsr_stats total{};
  int64_t inbox = n;
  if (hsr_status r = subcycle_resident(ctx, sp, n, f, ids, msk, &inbox, total)) return r;
  if (mem == HSR_MEM_HOST) {
    float *out[8] = {x, y, z, vx, vy, vz, mass, phi};
    for (int i = 0; i < 8; ++i)
      CU(cudaMemcpyAsync(out[i], f[i], size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H arrays");
    CU(cudaMemcpyAsync(id, ids, size_t(n) * 8, cudaMemcpyDeviceToHost, s), "D2H ids");
    CU(cudaMemcpyAsync(mask, msk, size_t(n) * 2, cudaMemcpyDeviceToHost, s), "D2H masks");
    total.h2d_bytes = n * 42;
    total.d2h_bytes = n * 42;
  }
  CU(cudaStreamSynchronize(s), "sub-cycle");
  if (n_inbox) *n_inbox = inbox;
  total.n = n;
  total.t_total_ms = ms_since(t_start);
  ctx->stats = total;
  ctx->have_lists = !sp->skip_kick && sp->nsub > 0;
  return HSR_OK;
}

}  // extern "C"

namespace {

// hsr_force_fwd (accumulate = false: dv written) and hsr_force_kick
// (accumulate = true: dv added into the arrays).
hsr_status force_fwd_impl(hsr_ctx *ctx, const hsr_params *p, int64_t n, const float *x,
                          const float *y, const float *z, const float *mass, float *dvx,
                          float *dvy, float *dvz, int32_t mem, bool accumulate) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t_start = clk::now();
  const void *arrs[10] = {x, y, z, dvx, dvy, dvz, mass, x, x, x};
  if (hsr_status e = check_params(p, n, arrs, ctx->err)) return e;
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  if (p->tree != HSR_TREE_RCB)
    return ctx->fail(HSR_ERR_UNSUPPORTED, "the forward/adjoint pair builds the RCB tree only");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->have_lists = false;
  ctx->tape = false;
  ctx->last_was_batch = false;
  ctx->tape_boxes = 0;
  cudaStream_t s = ctx->stream;
  const size_t nb = size_t(std::max<int64_t>(n, 1)) * 4;
  CU(ctx->d_pos4.ensure(size_t(std::max<int64_t>(n, 1)) * 16), "cudaMalloc(pos4)");
  const float *in[4] = {x, y, z, mass};
  if (mem == HSR_MEM_HOST) {
    CU(ctx->d_in.ensure(4 * nb + 1024), "cudaMalloc(in)");
    for (int i = 0; i < 4; ++i) {
      float *d = reinterpret_cast<float *>(ctx->d_in.as<char>() + i * ((nb + 255) & ~size_t(255)));
      CU(cudaMemcpyAsync(d, in[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D positions");
      in[i] = d;
    }
  }
  float4 *pos4 = ctx->d_pos4.as<float4>();
  CU(hsr::launch_pack4(in[0], in[1], in[2], in[3], pos4, n, s), "pack kernel");
  hsr::TreeConfig cfg{};
  for (int i = 0; i < 3; ++i) {
    cfg.min[i] = p->min[i];
    cfg.max[i] = p->max[i];
    cfg.min_force[i] = p->min_force[i];
    cfg.max_force[i] = p->max_force[i];
  }
  cfg.fsrrmax = p->fsrrmax;
  cfg.prune2 = cull2(cut2(p->law, p->fsrrmax));
  cfg.tan_oa = std::tan(p->open_angle);
  cfg.ppc = p->ppc;
  cfg.nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
  cfg.tdpts = p->tdpts;
  cfg.group = ctx->tune.group;  // the adjoint kernel takes groups of 16 or 32
  cudaError_t e = ctx->tree.build(cfg, n, pos4, kJSplit, s);
  if (e != cudaSuccess) {
    if (ctx->tree.error()) return ctx->fail(HSR_ERR_UNSUPPORTED, ctx->tree.error());
    return ctx->cuda_fail(e, "device tree build");
  }
  const hsr::DeviceTreeInfo &ti = ctx->tree.info();
  Work &w = ctx->work;
  set_work_params(w, p, n, ctx->tune);
  CU(ctx->d_vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4 + 256), "cudaMalloc(vel)");
  float *dv = ctx->d_vel.as<float>();
  CU(cudaMemsetAsync(dv, 0, size_t(3 * n) * 4, s), "zero dv");
  w.table = ctx->tree.table();
  w.leaves = ctx->tree.leaves();
  w.idx = ctx->tree.index();
  w.items = ctx->tree.items();
  w.gidx = ctx->tree.gidx();
  w.group = ctx->tree.group();
  w.vel = dv;
  w.nleaves = ti.processed_leaves;
  w.nitems = ti.items;
  w.device_built = true;
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(ctx->launch_pairs(w.kernel), "pair kernel");
  CU(cudaEventRecord(ctx->ev1, s), "event");
  // back to the caller's order
  CU(ctx->d_out.ensure(3 * nb + 1024), "cudaMalloc(out)");
  float *ob = ctx->d_out.as<float>();
  const size_t stride = ((nb + 255) & ~size_t(255)) / 4;
  float *outs[3] = {dvx, dvy, dvz};
  for (int d = 0; d < 3; ++d) {
    float *o = mem == HSR_MEM_HOST ? ob + d * stride : outs[d];
    if (accumulate) {
      if (mem == HSR_MEM_HOST)
        CU(cudaMemcpyAsync(o, outs[d], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D v");
      CU(hsr::launch_scatter_add_f32(dv + d * n, ctx->tree.perm(), o, n, s), "scatter-add dv");
    } else {
      CU(hsr::launch_scatter_f32(dv + d * n, ctx->tree.perm(), o, n, s), "scatter dv");
    }
    if (mem == HSR_MEM_HOST)
      CU(cudaMemcpyAsync(outs[d], o, size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H dv");
  }
  CU(cudaStreamSynchronize(s), "forward");
  float fms = 0;
  CU(cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1), "event time");
  hsr_stats st{};
  st.n = n;
  st.nodes = ti.nodes;
  st.processed_leaves = ti.processed_leaves;
  st.list_entries = ti.list_entries;
  st.pairs = ti.pairs;
  st.work_items = ti.items;
  st.cm_fallbacks = ti.cm_fallbacks;
  st.t_build_ms = ctx->tree.build_ms();
  st.t_walk_ms = ctx->tree.lists_ms();
  st.t_force_ms = fms;
  st.t_total_ms = ms_since(t_start);
  ctx->stats = st;
  ctx->have_lists = true;
  ctx->last_tdpts = p->tdpts;
  ctx->tape_nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
  ctx->tape_ppc = p->ppc;
  ctx->tape = true;
  return HSR_OK;
}

}  // namespace

extern "C" {

hsr_status hsr_force_fwd(hsr_ctx *ctx, const hsr_params *p, int64_t n, const float *x,
                         const float *y, const float *z, const float *mass, float *dvx,
                         float *dvy, float *dvz, int32_t mem) {
  return force_fwd_impl(ctx, p, n, x, y, z, mass, dvx, dvy, dvz, mem, false);
}

hsr_status hsr_force_kick(hsr_ctx *ctx, const hsr_params *p, int64_t n, const float *x,
                          const float *y, const float *z, const float *mass, float *vx,
                          float *vy, float *vz, int32_t mem) {
  return force_fwd_impl(ctx, p, n, x, y, z, mass, vx, vy, vz, mem, true);
}

hsr_status hsr_stream(hsr_ctx *ctx, int64_t n, float *x, float *y, float *z, const float *vx,
                      const float *vy, const float *vz, float alpha, float pp, float tau,
                      float adot, int32_t mem) {
  if (!ctx || n < 0 || (n > 0 && (!x || !y || !z || !vx || !vy || !vz))) return HSR_ERR_ARG;
  if (mem != HSR_MEM_DEVICE)
    return ctx->fail(HSR_ERR_UNSUPPORTED, "hsr_stream takes device arrays (HSR_MEM_DEVICE)");
  if (!(alpha != 0.0f) || !(adot != 0.0f) || !(pp > 0.0f))
    return ctx->fail(HSR_ERR_ARG, "alpha, adot must be nonzero and pp positive");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  // map1's prefactor in float, as the reference computes it
  const float pf = std::pow(pp, float(1.0 + 1.0 / alpha));
  const float prefactor = float(1.0 / (alpha * adot * pf));
  const float pt = prefactor * tau;
  CU(hsr::launch_stream(x, y, z, vx, vy, vz, n, pt, ctx->stream), "stream kernel");
  CU(cudaStreamSynchronize(ctx->stream), "stream kernel execution");
  return HSR_OK;
}

hsr_status hsr_force_vjp(hsr_ctx *ctx, const float *dvbx, const float *dvby, const float *dvbz,
                         float *xbx, float *xby, float *xbz, int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  if (!ctx->tape) return ctx->fail(HSR_ERR_STATE, "hsr_force_vjp needs a preceding hsr_force_fwd");
  const bool quad = ctx->last_tdpts == 12;
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  const Work &w = ctx->work;
  const int64_t n = w.n;
  if (n > 0 && (!dvbx || !dvby || !dvbz || !xbx || !xby || !xbz))
    return ctx->fail(HSR_ERR_ARG, "null array");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  const hsr::DeviceTreeInfo &ti = ctx->tree.info();
  const int64_t ntab = n + ti.nodes * ctx->last_tdpts;
  const size_t sn = size_t((std::max<int64_t>(n, 1) + 63) & ~int64_t(63));
  const size_t st_ = size_t((std::max<int64_t>(ntab, 1) + 63) & ~int64_t(63));
  const size_t sa = (size_t(std::max<int64_t>(ti.nodes, 1)) * 4 + 63) & ~size_t(63);
  // cotangent (caller order) | cotangent (tree order) | xbar table (3 x ntab) |
  // mass cotangents (ntab, 12-point pseudo-particles) | per node: xc and tdr
  // cotangents | error flag
  CU(ctx->d_adj.ensure((6 * sn + 4 * st_ + sa + 64) * 4), "cudaMalloc(adjoint)");
  float *ub = ctx->d_adj.as<float>();
  float *ut = ub + 3 * sn;
  float *xb = ut + 3 * sn;
  float *mbar = xb + 3 * st_;
  float *xcbar = mbar + st_;
  float *tdrbar = xcbar + 3 * std::max<int64_t>(ti.nodes, 1);
  float *acc = xcbar + sa;
  const float *uin[3] = {dvbx, dvby, dvbz};
  const int32_t *perm = ctx->tree.perm();
  for (int d = 0; d < 3; ++d) {
    const float *src = uin[d];
    if (mem == HSR_MEM_HOST) {
      CU(cudaMemcpyAsync(ub + d * sn, uin[d], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D cotangent");
      src = ub + d * sn;
    }
    CU(hsr::launch_gather_f32(src, perm, ut + d * sn, n, s), "gather cotangent");
  }
  CU(cudaMemsetAsync(xb, 0, (quad ? 4 : 3) * st_ * 4, s), "zero xbar");
  CU(ctx->d_queue.ensure(64), "cudaMalloc(queue)");
  CU(cudaMemsetAsync(ctx->d_queue.p, 0, 2 * sizeof(unsigned long long), s), "reset queue");
  if (ctx->batched_ctas == 0) ctx->batched_ctas = hsr::batched_resident_ctas(ctx->device);
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(hsr::launch_pairs_vjp(w.law, w.table, w.items, w.nitems, w.gidx, w.idx, ut, ut + sn, ut + 2 * sn,
                           xb, xb + st_, xb + 2 * st_, w.fcoeff, w.rsm2, w.rc2, w.rcull2,
                           ctx->d_queue.as<unsigned long long>(), ctx->batched_ctas, s,
                           quad ? mbar : nullptr, n),
     "adjoint kernel");
  int32_t *aerr = reinterpret_cast<int32_t *>(acc);
  CU(cudaMemsetAsync(aerr, 0, sizeof(int32_t), s), "reset flag");
  if (quad)
    CU(hsr::launch_pseudo_adjoint_quad(ctx->tree.nodes(), ctx->tree.levels(), w.table, n,
                                       ctx->tape_nd, ctx->tape_ppc, xb, xb + st_, xb + 2 * st_,
                                       mbar, xcbar, tdrbar, aerr, s),
       "pseudo-particle adjoint");
  else
    CU(hsr::launch_pseudo_adjoint(ctx->tree.nodes(), ctx->tree.levels(), w.table, n, xb, xb + st_,
                                  xb + 2 * st_, aerr, s),
       "pseudo-particle adjoint");
  CU(cudaEventRecord(ctx->ev1, s), "event");
  float *outs[3] = {xbx, xby, xbz};
  for (int d = 0; d < 3; ++d) {
    float *o = mem == HSR_MEM_HOST ? ub + d * sn : outs[d];
    CU(hsr::launch_scatter_f32(xb + d * st_, perm, o, n, s), "scatter xbar");
    if (mem == HSR_MEM_HOST)
      CU(cudaMemcpyAsync(outs[d], o, size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H xbar");
  }
  int32_t h_aerr = 0;
  CU(cudaMemcpyAsync(&h_aerr, aerr, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H flag");
  CU(cudaStreamSynchronize(s), "adjoint");
  if (h_aerr) return ctx->fail(HSR_ERR_STATE, "pseudo-particle adjoint: inconsistent tree");
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
  ctx->stats.t_force_ms = ms;
  return HSR_OK;
}

hsr_status hsr_last_perm(const hsr_ctx *ctx_c, int64_t *perm) {
  hsr_ctx *ctx = const_cast<hsr_ctx *>(ctx_c);
  if (!ctx || !perm) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  const int64_t n = ctx->work.n;
  if (!ctx->work.device_built) {
    const auto &el = ctx->host->elems();
    for (int64_t i = 0; i < n; ++i) perm[i] = el[i].idx;
    return HSR_OK;
  }
  std::vector<int32_t> p32(static_cast<size_t>(std::max<int64_t>(n, 1)));
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  CU(cudaMemcpy(p32.data(), ctx->tree.perm(), size_t(n) * 4, cudaMemcpyDeviceToHost), "D2H perm");
  for (int64_t i = 0; i < n; ++i) perm[i] = p32[i];
  return HSR_OK;
}

hsr_status hsr_tree_size(const hsr_ctx *ctx, int64_t *nnodes) {
  if (!ctx || !nnodes) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  *nnodes = ctx->work.device_built ? ctx->tree.info().nodes : ctx->host->num_nodes();
  return HSR_OK;
}

hsr_status hsr_tree_export(const hsr_ctx *ctx_c, int64_t *count, int64_t *offset, int64_t *cl,
                           int64_t *cr, float *tdr, float *bbox9, float *ppm) {
  hsr_ctx *ctx = const_cast<hsr_ctx *>(ctx_c);
  if (!ctx || !count || !offset || !cl || !cr || !tdr || !bbox9 || !ppm) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  const int k = ctx->last_tdpts;
  if (!ctx->work.device_built) {
    const auto &H = *ctx->host;
    for (int64_t t = 0; t < H.num_nodes(); ++t) {
      const hsr::Node &N = H.node(t);
      count[t] = N.count;
      offset[t] = N.offset;
      cl[t] = N.c[0];
      cr[t] = N.c[1];
      tdr[t] = N.tdr;
      for (int i = 0; i < 3; ++i) {
        bbox9[9 * t + i] = N.xmin[i];
        bbox9[9 * t + 3 + i] = N.xmax[i];
        bbox9[9 * t + 6 + i] = N.xc[i];
      }
      for (int i = 0; i < k; ++i) ppm[k * t + i] = N.ppm[i];
    }
    return HSR_OK;
  }
  const int64_t nn = ctx->tree.info().nodes;
  std::vector<hsr::DNode> nodes(static_cast<size_t>(std::max<int64_t>(nn, 1)));
  std::vector<float> pm(static_cast<size_t>(std::max<int64_t>(nn * k, 1)));
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  CU(cudaMemcpy(nodes.data(), ctx->tree.nodes(), size_t(nn) * sizeof(hsr::DNode), cudaMemcpyDeviceToHost),
     "D2H nodes");
  CU(cudaMemcpy(pm.data(), ctx->tree.ppm(), size_t(nn * k) * 4, cudaMemcpyDeviceToHost), "D2H ppm");
  for (int64_t t = 0; t < nn; ++t) {
    const hsr::DNode &N = nodes[t];
    count[t] = N.count;
    offset[t] = N.offset;
    cl[t] = N.cl;
    cr[t] = N.cr;
    tdr[t] = N.tdr;
    for (int i = 0; i < 3; ++i) {
      bbox9[9 * t + i] = N.xmin[i];
      bbox9[9 * t + 3 + i] = N.xmax[i];
      bbox9[9 * t + 6 + i] = N.xc[i];
    }
    for (int i = 0; i < k; ++i) ppm[k * t + i] = pm[k * t + i];
  }
  return HSR_OK;
}

hsr_status hsr_lists_export_index(const hsr_ctx *ctx_c, int64_t *entry_index) {
  hsr_ctx *ctx = const_cast<hsr_ctx *>(ctx_c);
  if (!ctx || !entry_index) return HSR_ERR_ARG;
  if (!ctx->have_lists) return HSR_ERR_STATE;
  if (!ctx->work.device_built) {
    export_lists(*ctx->host, ctx->h_pos.as<float>(), nullptr, nullptr, nullptr, nullptr, nullptr,
                 nullptr, nullptr, entry_index);
    return HSR_OK;
  }
  // the full lists from the segments (the device index array holds only the
  // entries the kernels need)
  const auto &ti = ctx->tree.info();
  const int64_t nl = ti.processed_leaves, ns = ti.segments;
  std::vector<hsr::LeafDesc> ld(static_cast<size_t>(std::max<int64_t>(nl, 1)));
  std::vector<hsr::SegDesc> sd(static_cast<size_t>(std::max<int64_t>(ns, 1)));
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  CU(cudaMemcpy(ld.data(), ctx->tree.leaves(), size_t(nl) * sizeof(hsr::LeafDesc),
                cudaMemcpyDeviceToHost), "D2H leaves");
  CU(cudaMemcpy(sd.data(), ctx->tree.segs(), size_t(ns) * sizeof(hsr::SegDesc),
                cudaMemcpyDeviceToHost), "D2H segments");
  int64_t seg = 0;
  for (int64_t l = 0; l < nl; ++l) {
    int64_t run = ld[l].list_begin;
    const int64_t end = ld[l].list_begin + ld[l].list_len;
    while (run < end && seg < ns) {
      const hsr::SegDesc &g = sd[seg++];
      for (int32_t q = 0; q < g.count; ++q) entry_index[run++] = int64_t(g.start) + q;
    }
  }
  return HSR_OK;
}

hsr_status hsr_rcb_kick_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                              const int64_t *ns, float *const *x, float *const *y,
                              float *const *z, float *const *vx, float *const *vy,
                              float *const *vz, float *const *mass, float *const *phi,
                              int64_t *const *id, uint16_t *const *mask, int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t_start = clk::now();
  if (nbox < 1 || nbox > (1 << 20) || !params || !ns || !x || !y || !z || !vx || !vy || !vz ||
      !mass || !phi || !id || !mask)
    return ctx->fail(HSR_ERR_ARG, "bad batch arguments");
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  for (int32_t b = 0; b < nbox; ++b) {
    const void *arrs[10] = {x[b], y[b], z[b], vx[b], vy[b], vz[b], mass[b], phi[b], id[b], mask[b]};
    if (hsr_status e = check_params(&params[b], ns[b], arrs, ctx->err)) return e;
    if (params[b].law != params[0].law)
      return ctx->fail(HSR_ERR_UNSUPPORTED, "all boxes of a batch use one force law");
    if (params[b].tree != HSR_TREE_RCB)
      return ctx->fail(HSR_ERR_UNSUPPORTED, "the multi-box kick builds RCB trees only");
  }
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->have_lists = false;
  ctx->tape = false;
  ctx->tape_boxes = 0;
  while (int32_t(ctx->boxes.size()) < nbox) ctx->boxes.emplace_back(new BoxState());
  hsr_stats st{};
  std::vector<hsr::BoxDesc> desc(static_cast<size_t>(nbox));
  int64_t total_items = 0;
  double build_ms = 0, lists_ms = 0;
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    if (!B.stream) CU(cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking), "box stream");
    if (!B.done) CU(cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming), "box event");
    B.status = HSR_OK;
    B.err.clear();
  }
  // One box: copies in, tree, lists, gathers, its descriptor; on the box's
  // own stream, errors into the box's status (the calls run on worker
  // threads).
  auto prepare_box = [&](int32_t b) {
    BoxState &B = *ctx->boxes[b];
    cudaStream_t s = B.stream;
    auto fail = [&](hsr_status code, const std::string &msg) {
      B.status = code;
      B.err = msg;
    };
#define BCU(call, what)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return fail(HSR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)
    BCU(cudaSetDevice(ctx->device), "cudaSetDevice");
    const hsr_params *p = &params[b];
    const int64_t n = ns[b];
    B.n = n;
    const ArrayLayout A(n);
    float *arr[8] = {x[b], y[b], z[b], vx[b], vy[b], vz[b], mass[b], phi[b]};
    BCU(B.out.ensure(A.bytes), "cudaMalloc(out)");
    BCU(B.pos4.ensure(size_t(std::max<int64_t>(n, 1)) * 16), "cudaMalloc(pos4)");
    BCU(B.vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4), "cudaMalloc(vel)");
    const float *in[8];
    const int64_t *in_id;
    const uint16_t *in_mask;
    if (mem == HSR_MEM_HOST) {
      BCU(B.in.ensure(A.bytes), "cudaMalloc(in)");
      char *ib = B.in.as<char>();
      for (int i = 0; i < 8; ++i) {
        BCU(cudaMemcpyAsync(ib + A.f[i], arr[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D arrays");
        in[i] = reinterpret_cast<const float *>(ib + A.f[i]);
      }
      BCU(cudaMemcpyAsync(ib + A.id, id[b], size_t(n) * 8, cudaMemcpyHostToDevice, s), "H2D ids");
      BCU(cudaMemcpyAsync(ib + A.mask, mask[b], size_t(n) * 2, cudaMemcpyHostToDevice, s), "H2D masks");
      in_id = reinterpret_cast<const int64_t *>(ib + A.id);
      in_mask = reinterpret_cast<const uint16_t *>(ib + A.mask);
    } else {
      for (int i = 0; i < 8; ++i) in[i] = arr[i];
      in_id = id[b];
      in_mask = mask[b];
    }
    BCU(hsr::launch_pack4(in[0], in[1], in[2], in[6], B.pos4.as<float4>(), n, s), "pack kernel");
    hsr::TreeConfig cfg{};
    for (int i = 0; i < 3; ++i) {
      cfg.min[i] = p->min[i];
      cfg.max[i] = p->max[i];
      cfg.min_force[i] = p->min_force[i];
      cfg.max_force[i] = p->max_force[i];
    }
    cfg.fsrrmax = p->fsrrmax;
    cfg.prune2 = cull2(cut2(p->law, p->fsrrmax));
    cfg.tan_oa = std::tan(p->open_angle);
    cfg.ppc = p->ppc;
    cfg.nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
    cfg.tdpts = p->tdpts;
    cfg.group = ctx->tune.group;
    cudaError_t e = B.tree.build(cfg, n, B.pos4.as<float4>(), kJSplit, s);
    if (e != cudaSuccess) {
      if (B.tree.error()) return fail(HSR_ERR_UNSUPPORTED, B.tree.error());
      return fail(HSR_ERR_CUDA, std::string("device tree build: ") + cudaGetErrorString(e));
    }
    const int32_t *perm = B.tree.perm();
    char *ob = B.out.as<char>();
    float *dv = B.vel.as<float>();
    BCU(hsr::launch_gather3_f32(in[3], in[4], in[5], perm, dv, n, s), "gather velocities");
    BCU(hsr::launch_outputs(B.tree.table(), in[7], in_id, in_mask, perm,
                            reinterpret_cast<float *>(ob + A.f[0]), reinterpret_cast<float *>(ob + A.f[1]),
                            reinterpret_cast<float *>(ob + A.f[2]), reinterpret_cast<float *>(ob + A.f[6]),
                            reinterpret_cast<float *>(ob + A.f[7]), reinterpret_cast<int64_t *>(ob + A.id),
                            reinterpret_cast<uint16_t *>(ob + A.mask), n, s),
        "gather outputs");
    BCU(cudaEventRecord(B.done, s), "box event");
#undef BCU
    hsr::BoxDesc &D = desc[b];
    D.table = B.tree.table();
    D.idx = B.tree.index();
    D.gidx = B.tree.gidx();
    D.vx = dv;
    D.vy = dv + n;
    D.vz = dv + 2 * n;
    D.fcoeff = p->fcoeff;
    D.rsm2 = p->rsm * p->rsm;
    D.rcut2 = cut2(p->law, p->fsrrmax);
    D.rcull2 = cull2(D.rcut2);
    D.law = hsr::make_law_s(p->law, D.rsm2, D.rcut2);
  };
  // Concurrent builds share no device state (the pseudo-particle design is a
  // read-only constant table), so boxes of any tdpts overlap.
  const int nthreads = int(std::min<int32_t>(nbox, kBatchThreads));
  if (nthreads <= 1) {
    for (int32_t b = 0; b < nbox; ++b) prepare_box(b);
  } else {
    std::atomic<int32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
      pool.emplace_back([&] {
        for (int32_t b; (b = next.fetch_add(1)) < nbox;) prepare_box(b);
      });
    for (auto &t : pool) t.join();
  }
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    if (B.status != HSR_OK) return ctx->fail(B.status, B.err);
    const hsr::DeviceTreeInfo &ti = B.tree.info();
    build_ms += B.tree.build_ms();
    lists_ms += B.tree.lists_ms();
    total_items += ti.items;
    st.n += B.n;
    st.nodes += ti.nodes;
    st.processed_leaves += ti.processed_leaves;
    st.list_entries += ti.list_entries;
    st.pairs += ti.pairs;
    st.cm_fallbacks += ti.cm_fallbacks;
    if (mem == HSR_MEM_HOST) st.h2d_bytes += B.n * 42;
    CU(cudaStreamWaitEvent(ctx->stream, B.done, 0), "wait for box");
  }
  cudaStream_t s = ctx->stream;
  // all boxes' items, tagged with their box, in one persistent launch
  CU(ctx->d_box_items.ensure(size_t(std::max<int64_t>(total_items, 1)) * sizeof(hsr::PairItem)),
     "cudaMalloc(items)");
  CU(ctx->d_box_desc.ensure(size_t(nbox) * sizeof(hsr::BoxDesc)), "cudaMalloc(boxes)");
  auto *items = ctx->d_box_items.as<hsr::PairItem>();
  int64_t at = 0;
  for (int32_t b = 0; b < nbox; ++b) {
    const int64_t ni = ctx->boxes[b]->tree.info().items;
    CU(hsr::launch_tag_items(ctx->boxes[b]->tree.items(), items + at, ni, b, s), "tag items");
    at += ni;
  }
  CU(cudaMemcpyAsync(ctx->d_box_desc.p, desc.data(), size_t(nbox) * sizeof(hsr::BoxDesc),
                     cudaMemcpyHostToDevice, s), "H2D box descriptors");
  CU(ctx->d_queue.ensure(64), "cudaMalloc(queue)");
  CU(cudaMemsetAsync(ctx->d_queue.p, 0, 2 * sizeof(unsigned long long), s), "reset queue");
  if (ctx->batched_ctas == 0) ctx->batched_ctas = hsr::batched_resident_ctas(ctx->device);
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(hsr::launch_pairs_batched_multi(params[0].law, ctx->tune.group, ctx->d_box_desc.as<hsr::BoxDesc>(), items,
                                     total_items, ctx->d_queue.as<unsigned long long>(),
                                     ctx->batched_ctas, s),
     "multi-box pair kernel");
  CU(cudaEventRecord(ctx->ev1, s), "event");
  const cudaMemcpyKind back = mem == HSR_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    const int64_t n = B.n;
    const ArrayLayout A(n);
    char *ob = B.out.as<char>();
    float *dv = B.vel.as<float>();
    float *arr[8] = {x[b], y[b], z[b], vx[b], vy[b], vz[b], mass[b], phi[b]};
    for (int d = 0; d < 3; ++d)
      CU(cudaMemcpyAsync(ob + A.f[3 + d], dv + d * n, size_t(n) * 4, cudaMemcpyDeviceToDevice, s),
         "copy velocities");
    for (int i = 0; i < 8; ++i)
      CU(cudaMemcpyAsync(arr[i], ob + A.f[i], size_t(n) * 4, back, s), "copy arrays back");
    CU(cudaMemcpyAsync(id[b], ob + A.id, size_t(n) * 8, back, s), "copy ids back");
    CU(cudaMemcpyAsync(mask[b], ob + A.mask, size_t(n) * 2, back, s), "copy masks back");
    if (mem == HSR_MEM_HOST) st.d2h_bytes += n * 42;
  }
  unsigned long long counters[2] = {0, 0};
  CU(cudaMemcpyAsync(counters, ctx->d_queue.p, sizeof(counters), cudaMemcpyDeviceToHost, s),
     "D2H counters");
  CU(cudaStreamSynchronize(s), "multi-box kick");
  float fms = 0;
  CU(cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1), "event time");
  st.t_force_ms = fms;
  st.t_build_ms = build_ms;
  st.t_walk_ms = lists_ms;
  st.evaluated_pairs = int64_t(counters[1]);
  st.work_items = total_items;
  st.kernel_launches = 1;
  st.t_total_ms = ms_since(t_start);
  ctx->stats = st;
  ctx->last_was_batch = true;
  ctx->batch_n = nbox;
  ctx->batch_items = total_items;
  ctx->batch_law = params[0].law;
  ctx->batch_group = ctx->tune.group;
  return HSR_OK;
}

}  // extern "C"

namespace {

// Runs the multi-box pair launch (queue reset + the persistent kernel over
// every box's items) as a CUDA graph: captured on each call and applied to
// the context's executable graph (cudaGraphExecUpdate), which is
// instantiated once and replayed.
cudaError_t launch_batch_graph(hsr_ctx *ctx, int law, int group, int64_t items) {
  cudaStream_t s = ctx->stream;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = cudaMemsetAsync(ctx->d_queue.p, 0, 2 * sizeof(unsigned long long), s);
  if (le == cudaSuccess)
    le = hsr::launch_pairs_batched_multi(law, group, ctx->d_box_desc.as<hsr::BoxDesc>(),
                                         ctx->d_box_items.as<hsr::PairItem>(), items,
                                         ctx->d_queue.as<unsigned long long>(), ctx->batched_ctas, s);
  e = cudaStreamEndCapture(s, &g);
  if (le != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return le != cudaSuccess ? le : e;
  }
  if (ctx->batch_exec) {
    cudaGraphExecUpdateResultInfo info{};
    if (cudaGraphExecUpdate(ctx->batch_exec, g, &info) != cudaSuccess) {
      cudaGetLastError();  // the topology changed: instantiate afresh
      cudaGraphExecDestroy(ctx->batch_exec);
      ctx->batch_exec = nullptr;
    }
  }
  if (!ctx->batch_exec) e = cudaGraphInstantiate(&ctx->batch_exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return e;
  return cudaGraphLaunch(ctx->batch_exec, s);
}

// hsr_force_fwd_batch (accumulate = false) and hsr_force_kick_batch
// (accumulate = true): every box's tree and lists built on the device (boxes
// prepared concurrently, each on its own stream), one persistent launch of the
// pair kernel over all boxes' items, dv back in each caller's order.  The
// boxes' trees stay as the tape of hsr_force_vjp_batch.
hsr_status force_batch_impl(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                            const int64_t *ns, const float *const *x, const float *const *y,
                            const float *const *z, const float *const *mass, float *const *dvx,
                            float *const *dvy, float *const *dvz, int32_t mem, bool accumulate) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t_start = clk::now();
  if (nbox < 1 || nbox > (1 << 20) || !params || !ns || !x || !y || !z || !mass || !dvx || !dvy ||
      !dvz)
    return ctx->fail(HSR_ERR_ARG, "bad batch arguments");
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  for (int32_t b = 0; b < nbox; ++b) {
    const void *arrs[10] = {x[b], y[b], z[b], dvx[b], dvy[b], dvz[b], mass[b], x[b], x[b], x[b]};
    if (hsr_status e = check_params(&params[b], ns[b], arrs, ctx->err)) return e;
    if (params[b].law != params[0].law)
      return ctx->fail(HSR_ERR_UNSUPPORTED, "all boxes of a batch use one force law");
    if (params[b].tree != HSR_TREE_RCB)
      return ctx->fail(HSR_ERR_UNSUPPORTED, "the multi-box forward builds RCB trees only");
  }
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->have_lists = false;
  ctx->tape = false;
  ctx->tape_boxes = 0;
  ctx->last_was_batch = false;
  while (int32_t(ctx->boxes.size()) < nbox) ctx->boxes.emplace_back(new BoxState());
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    if (!B.stream) CU(cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking), "box stream");
    if (!B.done) CU(cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming), "box event");
    B.status = HSR_OK;
    B.err.clear();
  }
  std::vector<hsr::BoxDesc> desc(static_cast<size_t>(nbox));
  auto prepare_box = [&](int32_t b) {
    BoxState &B = *ctx->boxes[b];
    cudaStream_t s = B.stream;
    auto fail = [&](hsr_status code, const std::string &msg) {
      B.status = code;
      B.err = msg;
    };
#define BCU(call, what)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return fail(HSR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)
    BCU(cudaSetDevice(ctx->device), "cudaSetDevice");
    const hsr_params *p = &params[b];
    const int64_t n = ns[b];
    B.n = n;
    const size_t nb = (size_t(std::max<int64_t>(n, 1)) * 4 + 255) & ~size_t(255);
    BCU(B.pos4.ensure(size_t(std::max<int64_t>(n, 1)) * 16), "cudaMalloc(pos4)");
    BCU(B.vel.ensure(size_t(std::max<int64_t>(3 * n, 1)) * 4), "cudaMalloc(vel)");
    const float *in[4] = {x[b], y[b], z[b], mass[b]};
    if (mem == HSR_MEM_HOST) {
      BCU(B.in.ensure(4 * nb), "cudaMalloc(in)");
      for (int i = 0; i < 4; ++i) {
        float *d = reinterpret_cast<float *>(B.in.as<char>() + i * nb);
        BCU(cudaMemcpyAsync(d, in[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D positions");
        in[i] = d;
      }
    }
    BCU(hsr::launch_pack4(in[0], in[1], in[2], in[3], B.pos4.as<float4>(), n, s), "pack kernel");
    hsr::TreeConfig cfg{};
    for (int i = 0; i < 3; ++i) {
      cfg.min[i] = p->min[i];
      cfg.max[i] = p->max[i];
      cfg.min_force[i] = p->min_force[i];
      cfg.max_force[i] = p->max_force[i];
    }
    cfg.fsrrmax = p->fsrrmax;
    cfg.prune2 = cull2(cut2(p->law, p->fsrrmax));
    cfg.tan_oa = std::tan(p->open_angle);
    cfg.ppc = p->ppc;
    cfg.nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
    cfg.tdpts = p->tdpts;
    cfg.group = ctx->tune.group;  // the adjoint kernel takes groups of 16 or 32
    cudaError_t e = B.tree.build(cfg, n, B.pos4.as<float4>(), kJSplit, s);
    if (e != cudaSuccess) {
      if (B.tree.error()) return fail(HSR_ERR_UNSUPPORTED, B.tree.error());
      return fail(HSR_ERR_CUDA, std::string("device tree build: ") + cudaGetErrorString(e));
    }
    float *dv = B.vel.as<float>();
    BCU(cudaMemsetAsync(dv, 0, size_t(3 * n) * 4, s), "zero dv");
    BCU(cudaEventRecord(B.done, s), "box event");
#undef BCU
    B.law = p->law;
    B.tdpts = p->tdpts;
    B.nd = int32_t(std::min<int64_t>(p->nd, INT32_MAX));
    B.ppc = p->ppc;
    B.fcoeff = p->fcoeff;
    B.rsm2 = p->rsm * p->rsm;
    B.rc2 = cut2(p->law, p->fsrrmax);
    B.rcull2 = cull2(B.rc2);
    hsr::BoxDesc &D = desc[b];
    D.table = B.tree.table();
    D.idx = B.tree.index();
    D.gidx = B.tree.gidx();
    D.vx = dv;
    D.vy = dv + n;
    D.vz = dv + 2 * n;
    D.fcoeff = B.fcoeff;
    D.rsm2 = B.rsm2;
    D.rcut2 = B.rc2;
    D.rcull2 = B.rcull2;
    D.law = hsr::make_law_s(p->law, D.rsm2, D.rcut2);
  };
  const int nthreads = int(std::min<int32_t>(nbox, kBatchThreads));
  if (nthreads <= 1) {
    for (int32_t b = 0; b < nbox; ++b) prepare_box(b);
  } else {
    std::atomic<int32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
      pool.emplace_back([&] {
        for (int32_t b; (b = next.fetch_add(1)) < nbox;) prepare_box(b);
      });
    for (auto &t : pool) t.join();
  }
  hsr_stats st{};
  int64_t total_items = 0;
  double build_ms = 0, lists_ms = 0;
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    if (B.status != HSR_OK) return ctx->fail(B.status, B.err);
    const hsr::DeviceTreeInfo &ti = B.tree.info();
    build_ms += B.tree.build_ms();
    lists_ms += B.tree.lists_ms();
    total_items += ti.items;
    st.n += B.n;
    st.nodes += ti.nodes;
    st.processed_leaves += ti.processed_leaves;
    st.list_entries += ti.list_entries;
    st.pairs += ti.pairs;
    st.cm_fallbacks += ti.cm_fallbacks;
    if (mem == HSR_MEM_HOST) st.h2d_bytes += B.n * 16 + (accumulate ? B.n * 12 : 0);
    CU(cudaStreamWaitEvent(ctx->stream, B.done, 0), "wait for box");
  }
  cudaStream_t s = ctx->stream;
  CU(ctx->d_box_items.ensure(size_t(std::max<int64_t>(total_items, 1)) * sizeof(hsr::PairItem)),
     "cudaMalloc(items)");
  CU(ctx->d_box_desc.ensure(size_t(nbox) * sizeof(hsr::BoxDesc)), "cudaMalloc(boxes)");
  auto *items = ctx->d_box_items.as<hsr::PairItem>();
  int64_t at = 0;
  for (int32_t b = 0; b < nbox; ++b) {
    const int64_t ni = ctx->boxes[b]->tree.info().items;
    CU(hsr::launch_tag_items(ctx->boxes[b]->tree.items(), items + at, ni, b, s), "tag items");
    at += ni;
  }
  CU(cudaMemcpyAsync(ctx->d_box_desc.p, desc.data(), size_t(nbox) * sizeof(hsr::BoxDesc),
                     cudaMemcpyHostToDevice, s), "H2D box descriptors");
  CU(ctx->d_queue.ensure(64), "cudaMalloc(queue)");
  if (ctx->batched_ctas == 0) ctx->batched_ctas = hsr::batched_resident_ctas(ctx->device);
  CU(cudaEventRecord(ctx->ev0, s), "event");
  if (total_items > 0)
    CU(launch_batch_graph(ctx, params[0].law, ctx->tune.group, total_items), "multi-box pair launch");
  CU(cudaEventRecord(ctx->ev1, s), "event");
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    const int64_t n = B.n;
    const size_t nb = (size_t(std::max<int64_t>(n, 1)) * 4 + 255) & ~size_t(255);
    float *dv = B.vel.as<float>();
    float *outs[3] = {dvx[b], dvy[b], dvz[b]};
    if (mem == HSR_MEM_HOST) CU(B.out.ensure(3 * nb), "cudaMalloc(out)");
    for (int d = 0; d < 3; ++d) {
      float *o = mem == HSR_MEM_HOST ? reinterpret_cast<float *>(B.out.as<char>() + d * nb) : outs[d];
      if (accumulate) {
        if (mem == HSR_MEM_HOST)
          CU(cudaMemcpyAsync(o, outs[d], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D v");
        CU(hsr::launch_scatter_add_f32(dv + d * n, B.tree.perm(), o, n, s), "scatter-add dv");
      } else {
        CU(hsr::launch_scatter_f32(dv + d * n, B.tree.perm(), o, n, s), "scatter dv");
      }
      if (mem == HSR_MEM_HOST)
        CU(cudaMemcpyAsync(outs[d], o, size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H dv");
    }
    if (mem == HSR_MEM_HOST) st.d2h_bytes += n * 12;
  }
  unsigned long long counters[2] = {0, 0};
  CU(cudaMemcpyAsync(counters, ctx->d_queue.p, sizeof(counters), cudaMemcpyDeviceToHost, s),
     "D2H counters");
  CU(cudaStreamSynchronize(s), "multi-box forward");
  float fms = 0;
  CU(cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1), "event time");
  st.t_force_ms = fms;
  st.t_build_ms = build_ms;
  st.t_walk_ms = lists_ms;
  st.evaluated_pairs = int64_t(counters[1]);
  st.work_items = total_items;
  st.kernel_launches = total_items > 0 ? 1 : 0;
  st.t_total_ms = ms_since(t_start);
  ctx->stats = st;
  ctx->tape_boxes = nbox;
  // the launch replays through hsr_bench_pairs as a multi-box kick's does
  ctx->last_was_batch = true;
  ctx->batch_n = nbox;
  ctx->batch_items = total_items;
  ctx->batch_law = params[0].law;
  ctx->batch_group = ctx->tune.group;
  return HSR_OK;
}

}  // namespace

extern "C" {

hsr_status hsr_force_fwd_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                               const int64_t *n, const float *const *x, const float *const *y,
                               const float *const *z, const float *const *mass, float *const *dvx,
                               float *const *dvy, float *const *dvz, int32_t mem) {
  return force_batch_impl(ctx, nbox, params, n, x, y, z, mass, dvx, dvy, dvz, mem, false);
}

hsr_status hsr_force_kick_batch(hsr_ctx *ctx, int32_t nbox, const hsr_params *params,
                                const int64_t *n, const float *const *x, const float *const *y,
                                const float *const *z, const float *const *mass, float *const *vx,
                                float *const *vy, float *const *vz, int32_t mem) {
  return force_batch_impl(ctx, nbox, params, n, x, y, z, mass, vx, vy, vz, mem, true);
}

hsr_status hsr_force_vjp_batch(hsr_ctx *ctx, int32_t nbox, const float *const *dvbx,
                               const float *const *dvby, const float *const *dvbz,
                               float *const *xbx, float *const *xby, float *const *xbz,
                               int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  if (ctx->tape_boxes < 1)
    return ctx->fail(HSR_ERR_STATE, "hsr_force_vjp_batch needs a preceding multi-box forward");
  if (nbox != ctx->tape_boxes)
    return ctx->fail(HSR_ERR_ARG, "the box count differs from the multi-box forward's");
  if (!dvbx || !dvby || !dvbz || !xbx || !xby || !xbz) return ctx->fail(HSR_ERR_ARG, "null array");
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  for (int32_t b = 0; b < nbox; ++b) {
    const BoxState &B = *ctx->boxes[b];
    if (B.n > 0 && (!dvbx[b] || !dvby[b] || !dvbz[b] || !xbx[b] || !xby[b] || !xbz[b]))
      return ctx->fail(HSR_ERR_ARG, "null array");
  }
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  std::vector<hsr::VjpBoxDesc> desc(static_cast<size_t>(nbox));
  bool any_quad = false;
  // per box: cotangent (caller order, host input) | cotangent (tree order) |
  // xbar table | mass cotangents (12-point boxes) | per node: xc and tdr
  // cotangents | error flag
  struct AdjLayout {
    size_t sn, st, sa;
  };
  auto layout = [](const BoxState &B) {
    const hsr::DeviceTreeInfo &ti = B.tree.info();
    const int64_t ntab = B.n + ti.nodes * B.tdpts;
    AdjLayout L;
    L.sn = size_t((std::max<int64_t>(B.n, 1) + 63) & ~int64_t(63));
    L.st = size_t((std::max<int64_t>(ntab, 1) + 63) & ~int64_t(63));
    L.sa = (size_t(std::max<int64_t>(ti.nodes, 1)) * 4 + 63) & ~size_t(63);
    return L;
  };
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    const int64_t n = B.n;
    const bool quad = B.tdpts == 12;
    any_quad = any_quad || quad;
    const AdjLayout AL = layout(B);
    const size_t sn = AL.sn, st_ = AL.st;
    CU(B.adj.ensure((6 * sn + 4 * st_ + AL.sa + 64) * 4), "cudaMalloc(adjoint)");
    float *ub = B.adj.as<float>();
    float *ut = ub + 3 * sn;
    float *xb = ut + 3 * sn;
    const float *uin[3] = {dvbx[b], dvby[b], dvbz[b]};
    for (int d = 0; d < 3; ++d) {
      const float *src = uin[d];
      if (mem == HSR_MEM_HOST) {
        CU(cudaMemcpyAsync(ub + d * sn, uin[d], size_t(n) * 4, cudaMemcpyHostToDevice, s),
           "H2D cotangent");
        src = ub + d * sn;
      }
      CU(hsr::launch_gather_f32(src, B.tree.perm(), ut + d * sn, n, s), "gather cotangent");
    }
    CU(cudaMemsetAsync(xb, 0, (quad ? 4 : 3) * st_ * 4, s), "zero xbar");
    hsr::VjpBoxDesc &D = desc[b];
    D.mb = quad ? xb + 3 * st_ : nullptr;
    D.npart = n;
    D.table = B.tree.table();
    D.idx = B.tree.index();
    D.gidx = B.tree.gidx();
    D.ux = ut;
    D.uy = ut + sn;
    D.uz = ut + 2 * sn;
    D.xbx = xb;
    D.xby = xb + st_;
    D.xbz = xb + 2 * st_;
    D.fcoeff = B.fcoeff;
    D.rsm2 = B.rsm2;
    D.rcut2 = B.rc2;
    D.rcull2 = B.rcull2;
  }
  CU(ctx->d_vjp_desc.ensure(size_t(nbox) * sizeof(hsr::VjpBoxDesc)), "cudaMalloc(vjp boxes)");
  CU(cudaMemcpyAsync(ctx->d_vjp_desc.p, desc.data(), size_t(nbox) * sizeof(hsr::VjpBoxDesc),
                     cudaMemcpyHostToDevice, s), "H2D vjp box descriptors");
  CU(ctx->d_queue.ensure(64), "cudaMalloc(queue)");
  CU(cudaMemsetAsync(ctx->d_queue.p, 0, 2 * sizeof(unsigned long long), s), "reset queue");
  if (ctx->batched_ctas == 0) ctx->batched_ctas = hsr::batched_resident_ctas(ctx->device);
  CU(cudaEventRecord(ctx->ev0, s), "event");
  CU(hsr::launch_pairs_vjp_multi(ctx->boxes[0]->law, ctx->d_vjp_desc.as<hsr::VjpBoxDesc>(),
                                 ctx->d_box_items.as<hsr::PairItem>(), ctx->batch_items,
                                 ctx->d_queue.as<unsigned long long>(), ctx->batched_ctas, s,
                                 any_quad),
     "multi-box adjoint kernel");
  CU(cudaEventRecord(ctx->ev1, s), "event");
  std::vector<int32_t *> aerrs;
  for (int32_t b = 0; b < nbox; ++b) {
    BoxState &B = *ctx->boxes[b];
    const int64_t n = B.n;
    const AdjLayout AL = layout(B);
    const size_t sn = AL.sn, st_ = AL.st;
    float *ub = B.adj.as<float>();
    float *xb = ub + 6 * sn;
    float *mbar = xb + 3 * st_, *xcbar = mbar + st_;
    float *tdrbar = xcbar + 3 * std::max<int64_t>(B.tree.info().nodes, 1);
    int32_t *aerr = reinterpret_cast<int32_t *>(xcbar + AL.sa);
    CU(cudaMemsetAsync(aerr, 0, sizeof(int32_t), s), "reset flag");
    if (B.tdpts == 12)
      CU(hsr::launch_pseudo_adjoint_quad(B.tree.nodes(), B.tree.levels(), B.tree.table(), n, B.nd,
                                         B.ppc, xb, xb + st_, xb + 2 * st_, mbar, xcbar, tdrbar,
                                         aerr, s),
         "pseudo-particle adjoint");
    else
      CU(hsr::launch_pseudo_adjoint(B.tree.nodes(), B.tree.levels(), B.tree.table(), n, xb,
                                    xb + st_, xb + 2 * st_, aerr, s),
         "pseudo-particle adjoint");
    aerrs.push_back(aerr);
    float *outs[3] = {xbx[b], xby[b], xbz[b]};
    for (int d = 0; d < 3; ++d) {
      float *o = mem == HSR_MEM_HOST ? ub + d * sn : outs[d];
      CU(hsr::launch_scatter_f32(xb + d * st_, B.tree.perm(), o, n, s), "scatter xbar");
      if (mem == HSR_MEM_HOST)
        CU(cudaMemcpyAsync(outs[d], o, size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H xbar");
    }
  }
  std::vector<int32_t> h_aerrs(aerrs.size(), 0);
  for (size_t b = 0; b < aerrs.size(); ++b)
    CU(cudaMemcpyAsync(&h_aerrs[b], aerrs[b], sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H flag");
  CU(cudaStreamSynchronize(s), "multi-box adjoint");
  for (int32_t e : h_aerrs)
    if (e) return ctx->fail(HSR_ERR_STATE, "pseudo-particle adjoint: inconsistent tree");
  float ms = 0;
  CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
  ctx->stats.t_force_ms = ms;
  return HSR_OK;
}

hsr_status hsr_build_lists(const hsr_params *p, int64_t n, float *x, float *y, float *z, float *vx,
                           float *vy, float *vz, float *mass, float *phi, int64_t *id, uint16_t *mask,
                           hsr_lists **out) {
  if (!out) return HSR_ERR_ARG;
  *out = nullptr;
  std::string err;
  const void *arrs[10] = {x, y, z, vx, vy, vz, mass, phi, id, mask};
  if (hsr_status e = check_params(p, n, arrs, err)) return e;
  auto *L = new (std::nothrow) hsr_lists();
  if (!L) return HSR_ERR_NOMEM;
  int nth = int(std::thread::hardware_concurrency());
  L->host.reset(new hsr::RcbHost(std::max(1, nth)));
  const PlanSizes ps = host_build(*L->host, p, n, x, y, z, mass, L->st);
  L->tab.resize(size_t(std::max<int64_t>(ps.ntab, 1)) * 4);
  std::vector<hsr::LeafDesc> ld(static_cast<size_t>(std::max<int64_t>(ps.nleaves, 1)));
  std::vector<hsr::SegDesc> sd(static_cast<size_t>(std::max<int64_t>(ps.nsegs, 1)));
  std::vector<int64_t> list_begin;
  host_fill(*L->host, n, x, y, z, vx, vy, vz, mass, phi, id, mask, L->tab.data(), nullptr, ld.data(),
            sd.data(), &list_begin);
  std::vector<int32_t> gidx;
  std::vector<hsr::PairItem> items;
  make_items(*L->host, list_begin, kJSplit, 32, gidx, items);
  L->st.work_items = int64_t(items.size());
  *out = L;
  return HSR_OK;
}

hsr_status hsr_lists_info(const hsr_lists *L, int64_t *nleaves, int64_t *nentries, hsr_stats *st) {
  if (!L) return HSR_ERR_ARG;
  if (nleaves) *nleaves = int64_t(L->host->leaves().size());
  if (nentries) *nentries = L->host->list_entries();
  if (st) *st = L->st;
  return HSR_OK;
}

hsr_status hsr_lists_get(const hsr_lists *L, int64_t *leaf_offset, int64_t *leaf_count,
                         int64_t *list_ptr, float *ex, float *ey, float *ez, float *em) {
  if (!L || !leaf_offset || !leaf_count || !list_ptr || !ex || !ey || !ez || !em) return HSR_ERR_ARG;
  export_lists(*L->host, L->tab.data(), leaf_offset, leaf_count, list_ptr, ex, ey, ez, em, nullptr);
  return HSR_OK;
}

hsr_status hsr_lists_index(const hsr_lists *L, int64_t *entry_index) {
  if (!L || !entry_index) return HSR_ERR_ARG;
  export_lists(*L->host, L->tab.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
               entry_index);
  return HSR_OK;
}

hsr_status hsr_lists_free(hsr_lists *L) {
  if (!L) return HSR_ERR_ARG;
  delete L;
  return HSR_OK;
}

hsr_status hsr_force_law(hsr_ctx *ctx, int32_t law, float rsm, float fsrrmax, int64_t n,
                         const float *r2, float *g) {
  if (!ctx) return HSR_ERR_ARG;
  if (n < 0 || (n > 0 && (!r2 || !g))) return ctx->fail(HSR_ERR_ARG, "bad arrays");
  if (law != HSR_LAW_POLY6 && law != HSR_LAW_POLY5_STEP16) return ctx->fail(HSR_ERR_ARG, "unknown law");
  if (n == 0) return HSR_OK;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  CU(ctx->d_law.ensure(size_t(n) * 8), "cudaMalloc(law)");
  float *d = ctx->d_law.as<float>();
  cudaStream_t s = ctx->stream;
  CU(cudaMemcpyAsync(d, r2, size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D r2");
  CU(hsr::launch_force_law(law, d, d + n, n, rsm * rsm, cut2(law, fsrrmax), s), "law kernel");
  CU(cudaMemcpyAsync(g, d + n, size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H g");
  CU(cudaStreamSynchronize(s), "law kernel execution");
  return HSR_OK;
}

hsr_status hsr_bench_pairs(hsr_ctx *ctx, int32_t kernel, int32_t iters, int32_t flush_l2,
                           double *ms_per_launch) {
  if (!ctx || !ms_per_launch || iters < 1) return HSR_ERR_ARG;
  if (!ctx->have_lists && !ctx->last_was_batch) return ctx->fail(HSR_ERR_STATE, "no kick to replay");
  // replays run the kick's own kernel unless the plain one is asked for
  const bool multi = ctx->last_was_batch;
  if (multi && kernel == HSR_KERNEL_PLAIN)
    return ctx->fail(HSR_ERR_STATE, "a multi-box kick replays its batched launch only");
  const int kk = kernel == HSR_KERNEL_PLAIN ? HSR_KERNEL_PLAIN : ctx->work.kernel;
  if (!multi && kk == HSR_KERNEL_BATCHED && ctx->work.nitems == 0 && ctx->work.nleaves > 0)
    return ctx->fail(HSR_ERR_STATE, "last kick had no batched work to replay");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  const size_t flush_bytes = size_t(256) << 20;
  if (flush_l2) CU(ctx->d_flush.ensure(flush_bytes), "cudaMalloc(flush)");
  double total = 0;
  for (int it = 0; it < iters; ++it) {
    if (flush_l2) CU(cudaMemsetAsync(ctx->d_flush.p, it & 0xff, flush_bytes, s), "L2 flush");
    CU(cudaEventRecord(ctx->ev0, s), "event");
    CU(multi ? ctx->launch_batch_pairs() : ctx->launch_pairs(kk), "pair kernel");
    CU(cudaEventRecord(ctx->ev1, s), "event");
    CU(cudaEventSynchronize(ctx->ev1), "pair kernel execution");
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
    total += ms;
  }
  *ms_per_launch = total / iters;
  return HSR_OK;
}

hsr_status hsr_bench_pairs_graph(hsr_ctx *ctx, int32_t iters, int32_t flush_l2,
                                 double *ms_per_launch) {
  if (!ctx || !ms_per_launch || iters < 1) return HSR_ERR_ARG;
  if (!ctx->have_lists && !ctx->last_was_batch) return ctx->fail(HSR_ERR_STATE, "no kick to replay");
  const bool multi = ctx->last_was_batch;
  if (!multi && ctx->work.kernel != HSR_KERNEL_BATCHED)
    return ctx->fail(HSR_ERR_STATE, "graph replays run the batched kernel");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  CU(ctx->d_queue.ensure(64), "cudaMalloc(queue)");
  if (ctx->batched_ctas == 0) ctx->batched_ctas = hsr::batched_resident_ctas(ctx->device);
  const size_t flush_bytes = size_t(256) << 20;
  if (flush_l2) CU(ctx->d_flush.ensure(flush_bytes), "cudaMalloc(flush)");
  // capture the launch sequence (queue reset + persistent kernel) once
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = multi ? ctx->launch_batch_pairs() : ctx->launch_pairs(HSR_KERNEL_BATCHED);
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (le != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return ctx->cuda_fail(le, "capture pair launch");
  }
  CU(ce, "end capture");
  cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  CU(ie, "instantiate graph");
  double total = 0;
  cudaError_t e = cudaSuccess;
  for (int it = 0; it < iters && e == cudaSuccess; ++it) {
    if (flush_l2) e = cudaMemsetAsync(ctx->d_flush.p, it & 0xff, flush_bytes, s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev0, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    total += ms;
  }
  cudaGraphExecDestroy(exec);
  CU(e, "graph replay");
  *ms_per_launch = total / iters;
  return HSR_OK;
}

hsr_status hsr_set_tune(hsr_ctx *ctx, const hsr_tune *t) {
  if (!ctx || !t) return HSR_ERR_ARG;
  if (t->kernel != HSR_KERNEL_PLAIN && t->kernel != HSR_KERNEL_BATCHED)
    return ctx->fail(HSR_ERR_ARG, "tune.kernel must be HSR_KERNEL_PLAIN or HSR_KERNEL_BATCHED");
  if (t->leaf_threads != 32 && t->leaf_threads != 64 && t->leaf_threads != 128)
    return ctx->fail(HSR_ERR_ARG, "tune.leaf_threads must be 32, 64 or 128");
  if (t->group != 16 && t->group != 32) return ctx->fail(HSR_ERR_ARG, "tune.group must be 16 or 32");
  ctx->tune = *t;
  ctx->tune.reserved = 0;
  return HSR_OK;
}

hsr_status hsr_get_tune(const hsr_ctx *ctx, hsr_tune *t) {
  if (!ctx || !t) return HSR_ERR_ARG;
  *t = ctx->tune;
  return HSR_OK;
}

hsr_status hsr_autotune(hsr_ctx *ctx, int32_t iters, int32_t flush_l2, hsr_tune_row *rows,
                        int32_t cap, int32_t *nrows) {
  if (!ctx || iters < 1 || cap < 0 || (cap > 0 && !rows)) return HSR_ERR_ARG;
  if (!ctx->have_lists || !ctx->work.device_built || ctx->last_was_batch)
    return ctx->fail(HSR_ERR_STATE, "autotune replays the last single-box kick built on the device");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  Work &w = ctx->work;
  const int saved_kernel = w.kernel, saved_threads = w.leaf_threads, saved_group = w.group;
  std::vector<hsr_tune_row> table;
  auto time_shape = [&](const hsr_tune &t) -> hsr_status {
    w.kernel = t.kernel;
    w.leaf_threads = t.leaf_threads;
    w.group = t.group;
    double warm = 0, ms = 0;
    if (hsr_status r = hsr_bench_pairs(ctx, t.kernel, 1, flush_l2, &warm)) return r;
    if (hsr_status r = hsr_bench_pairs(ctx, t.kernel, iters, flush_l2, &ms)) return r;
    int64_t ev = ctx->tree.padded_pairs();
    if (t.kernel == HSR_KERNEL_BATCHED) {
      unsigned long long c[2] = {0, 0};
      CU(cudaMemcpy(c, ctx->d_queue.p, sizeof(c), cudaMemcpyDeviceToHost), "D2H counters");
      ev = int64_t(c[1]);
    }
    table.push_back(hsr_tune_row{t, ms, ev});
    return HSR_OK;
  };
  hsr_status r = HSR_OK;
  for (int nt : {32, 64, 128})
    if (r == HSR_OK) r = time_shape(hsr_tune{HSR_KERNEL_PLAIN, nt, saved_group, 0});
  for (int g : {16, 32}) {
    if (r != HSR_OK) break;
    if (ctx->tree.regroup(g, kJSplit, ctx->stream) != cudaSuccess) {
      r = ctx->fail(HSR_ERR_CUDA, "regroup");
      break;
    }
    w.items = ctx->tree.items();
    w.gidx = ctx->tree.gidx();
    w.nitems = ctx->tree.info().items;
    r = time_shape(hsr_tune{HSR_KERNEL_BATCHED, saved_threads, g, 0});
  }
  if (r != HSR_OK) {
    w.kernel = saved_kernel;
    w.leaf_threads = saved_threads;
    w.group = saved_group;
    return r;
  }
  // the context takes the fastest shape
  size_t best = 0;
  for (size_t i = 1; i < table.size(); ++i)
    if (table[i].ms < table[best].ms) best = i;
  hsr_tune t = table[best].tune;
  // each family keeps its own best shape for explicit kernel requests
  double bp = 1e300, bb = 1e300;
  for (const auto &row : table) {
    if (row.tune.kernel == HSR_KERNEL_PLAIN && row.ms < bp) bp = row.ms, t.leaf_threads = row.tune.leaf_threads;
    if (row.tune.kernel == HSR_KERNEL_BATCHED && row.ms < bb) bb = row.ms, t.group = row.tune.group;
  }
  ctx->tune = t;
  if (ctx->tree.regroup(t.group, kJSplit, ctx->stream) != cudaSuccess)
    return ctx->fail(HSR_ERR_CUDA, "regroup");
  w.items = ctx->tree.items();
  w.gidx = ctx->tree.gidx();
  w.nitems = ctx->tree.info().items;
  w.kernel = t.kernel;
  w.leaf_threads = t.leaf_threads;
  w.group = t.group;
  const int32_t nr = int32_t(table.size());
  for (int32_t i = 0; i < std::min(nr, cap); ++i) rows[i] = table[size_t(i)];
  if (nrows) *nrows = nr;
  return HSR_OK;
}

hsr_status hsr_pairs_in_cutoff(hsr_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return HSR_ERR_ARG;
  const Work &w = ctx->work;
  if (!ctx->have_lists || !w.device_built || ctx->last_was_batch)
    return ctx->fail(HSR_ERR_STATE, "hsr_pairs_in_cutoff needs a single-box kick built on the device");
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  CU(ctx->d_queue.ensure(64), "cudaMalloc(counter)");
  unsigned long long *c = ctx->d_queue.as<unsigned long long>() + 4;
  CU(cudaMemsetAsync(c, 0, sizeof(unsigned long long), s), "counter clear");
  CU(hsr::launch_count_in_cutoff(w.table, w.leaves, w.nleaves, w.idx, w.rc2, c, s), "count kernel");
  unsigned long long h = 0;
  CU(cudaMemcpyAsync(&h, c, sizeof(h), cudaMemcpyDeviceToHost, s), "count copy");
  CU(cudaStreamSynchronize(s), "count");
  *count = int64_t(h);
  return HSR_OK;
}

hsr_status hsr_probe_fp32_peak(hsr_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return HSR_ERR_ARG;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  int sms = 0;
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device), "device attribute");
  const int threads = 512, blocks = sms * 4, iters = 1 << 16;
  CU(ctx->d_probe.ensure(size_t(blocks) * threads * 4), "cudaMalloc(probe)");
  cudaStream_t s = ctx->stream;
  CU(hsr::launch_ffma_probe(ctx->d_probe.as<float>(), blocks, threads, 256, s), "probe warm-up");
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    CU(cudaEventRecord(ctx->ev0, s), "event");
    CU(hsr::launch_ffma_probe(ctx->d_probe.as<float>(), blocks, threads, iters, s), "probe");
    CU(cudaEventRecord(ctx->ev1, s), "event");
    CU(cudaEventSynchronize(ctx->ev1), "probe execution");
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
    const double flops = 2.0 * 8.0 * double(iters) * double(blocks) * threads;
    best = std::max(best, flops / (double(ms) * 1e-3) / 1e12);
  }
  *tflops = best;
  return HSR_OK;
}

}  // extern "C"

// ---- long-range PM kick (hacc_pm.h) -------------------------------------

namespace {

hsr_status pm_check(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const void *const *arrs,
                    int narr, int32_t mem) {
  if (!p) return ctx->fail(HSR_ERR_ARG, "null PM params");
  if (n < 0) return ctx->fail(HSR_ERR_ARG, "negative particle count");
  if (n > 0)
    for (int i = 0; i < narr; ++i)
      if (!arrs[i]) return ctx->fail(HSR_ERR_ARG, "null particle array");
  if (p->ng < 2 || (p->ng & 1) || p->ng > 4096)
    return ctx->fail(HSR_ERR_ARG, "ng must be even and in [2, 4096]");
  // GridExchange fills the ngo + 1 upper dead cells from the alive block
  if (p->ngo < 0 || p->ngo >= p->ng) return ctx->fail(HSR_ERR_ARG, "ngo must be in [0, ng)");
  if (p->precision != HSR_PM_F64 && p->precision != HSR_PM_F32)
    return ctx->fail(HSR_ERR_ARG, "unknown PM precision");
  if (mem != HSR_MEM_HOST && mem != HSR_MEM_DEVICE) return ctx->fail(HSR_ERR_ARG, "bad memory kind");
  return HSR_OK;
}

hsr_pm::Params pm_params(const hsr_pm_params *p) {
  hsr_pm::Params q;
  q.ng = p->ng;
  q.ngo = p->ngo;
  q.gpscal = p->gpscal;
  q.fscal = p->fscal;
  q.tau = p->tau;
  q.prec = p->precision == HSR_PM_F32 ? hsr_pm::PREC_F32 : hsr_pm::PREC_F64;
  return q;
}

hsr_status pm_prepare(hsr_ctx *ctx, const hsr_pm::Params &q) {
  if (!ctx->pm) ctx->pm.reset(new (std::nothrow) hsr_pm::Solver());
  if (!ctx->pm) return ctx->fail(HSR_ERR_NOMEM, "PM solver");
  std::string err;
  if (!ctx->pm->prepare(q.ng, q.prec, ctx->stream, &err)) return ctx->fail(HSR_ERR_CUDA, err);
  return HSR_OK;
}

}  // namespace

extern "C" {

hsr_status hsr_pm_tables(int32_t ng, double *filter, double *denom, double *gradient) {
  if (ng < 2 || (ng & 1) || !filter || !denom || !gradient) return HSR_ERR_ARG;
  hsr_pm::quiet_tables(ng, filter, denom, gradient);
  return HSR_OK;
}

hsr_status hsr_pm_kick(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                       const float *y, const float *z, float *vx, float *vy, float *vz,
                       int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t0 = clk::now();
  const void *arrs[6] = {x, y, z, vx, vy, vz};
  hsr_status st = pm_check(ctx, p, n, arrs, 6, mem);
  if (st != HSR_OK) return st;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  const hsr_pm::Params q = pm_params(p);
  if ((st = pm_prepare(ctx, q)) != HSR_OK) return st;
  cudaStream_t s = ctx->stream;
  hsr_pm_stats ps{};
  const float *dx = x, *dy = y, *dz = z;
  float *dvx = vx, *dvy = vy, *dvz = vz;
  const size_t nb = size_t(n) * sizeof(float);
  if (mem == HSR_MEM_HOST && n > 0) {
    CU(ctx->d_pm.ensure(6 * nb), "cudaMalloc(PM particles)");
    float *b = ctx->d_pm.as<float>();
    dx = b;
    dy = b + n;
    dz = b + 2 * n;
    dvx = b + 3 * n;
    dvy = b + 4 * n;
    dvz = b + 5 * n;
    CU(cudaEventRecord(ctx->ev0, s), "event");
    const float *src[6] = {x, y, z, vx, vy, vz};
    for (int a = 0; a < 6; ++a)
      CU(cudaMemcpyAsync(b + a * n, src[a], nb, cudaMemcpyHostToDevice, s), "PM copy in");
    CU(cudaEventRecord(ctx->ev1, s), "event");
    CU(cudaEventSynchronize(ctx->ev1), "PM copy in");
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ps.t_h2d_ms = ms;
    ps.h2d_bytes = int64_t(6 * nb);
  }
  cudaEvent_t ev[4] = {ctx->ev0, ctx->ev1, ctx->ev2, ctx->ev3};
  hsr_pm::Timing tm;
  std::string err;
  if (!ctx->pm->kick(q, n, dx, dy, dz, dvx, dvy, dvz, s, ev, &tm, &err))
    return ctx->fail(HSR_ERR_CUDA, err);
  if (mem == HSR_MEM_HOST && n > 0) {
    CU(cudaEventRecord(ctx->ev0, s), "event");
    float *dst[3] = {vx, vy, vz};
    for (int a = 0; a < 3; ++a)
      CU(cudaMemcpyAsync(dst[a], ctx->d_pm.as<float>() + (3 + a) * n, nb, cudaMemcpyDeviceToHost, s),
         "PM copy out");
    CU(cudaEventRecord(ctx->ev1, s), "event");
    CU(cudaEventSynchronize(ctx->ev1), "PM copy out");
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ps.t_d2h_ms = ms;
    ps.d2h_bytes = int64_t(3 * nb);
  }
  ps.t_deposit_ms = tm.deposit_ms;
  ps.t_solve_ms = tm.solve_ms;
  ps.t_interp_ms = tm.interp_ms;
  ps.kernel_launches = tm.launches;
  ps.fft_execs = tm.fft_execs;
  ps.t_total_ms = ms_since(t0);
  ctx->pm_stats = ps;
  return HSR_OK;
}

hsr_status hsr_pm_fields(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                         const float *y, const float *z, float *rho, float *grad, int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  const void *arrs[3] = {x, y, z};
  hsr_status st = pm_check(ctx, p, n, arrs, 3, mem);
  if (st != HSR_OK) return st;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  const hsr_pm::Params q = pm_params(p);
  if ((st = pm_prepare(ctx, q)) != HSR_OK) return st;
  cudaStream_t s = ctx->stream;
  const float *dx = x, *dy = y, *dz = z;
  const size_t nb = size_t(n) * sizeof(float);
  if (mem == HSR_MEM_HOST && n > 0) {
    CU(ctx->d_pm.ensure(3 * nb), "cudaMalloc(PM particles)");
    float *b = ctx->d_pm.as<float>();
    const float *src[3] = {x, y, z};
    for (int a = 0; a < 3; ++a)
      CU(cudaMemcpyAsync(b + a * n, src[a], nb, cudaMemcpyHostToDevice, s), "PM copy in");
    dx = b;
    dy = b + n;
    dz = b + 2 * n;
  }
  std::string err;
  if (!ctx->pm->deposit(q, n, dx, dy, dz, s, &err)) return ctx->fail(HSR_ERR_CUDA, err);
  if (grad && !ctx->pm->solve(s, &err)) return ctx->fail(HSR_ERR_CUDA, err);
  if (!ctx->pm->export_fields(rho, grad, mem == HSR_MEM_HOST, s, &err))
    return ctx->fail(HSR_ERR_CUDA, err);
  return HSR_OK;
}

hsr_status hsr_treepm_step(hsr_ctx *ctx, const hsr_treepm_params *tp, int64_t n, float *x,
                           float *y, float *z, float *vx, float *vy, float *vz, float *mass,
                           float *phi, int64_t *id, uint16_t *mask, int32_t mem,
                           int64_t *n_inbox) {
  if (!ctx) return HSR_ERR_ARG;
  if (!tp) return ctx->fail(HSR_ERR_ARG, "null parameters");
  const auto t_start = clk::now();
  const hsr_subcycle_params *sp = &tp->sub;
  const void *arrs[10] = {x, y, z, vx, vy, vz, mass, phi, id, mask};
  if (hsr_status e = check_params(&sp->kick, n, arrs, ctx->err)) return e;
  if (sp->kick.tree != HSR_TREE_RCB)
    return ctx->fail(HSR_ERR_UNSUPPORTED, "the device sub-cycle builds the RCB tree only");
  if (sp->nsub < 0 || sp->ng[0] < 1 || sp->ng[1] < 1 || sp->ng[2] < 1 ||
      double(sp->ng[0]) * sp->ng[1] * sp->ng[2] >= 4294967295.0)
    return ctx->fail(HSR_ERR_ARG, "bad sub-cycle count or grid");
  const bool open = tp->pm_open.tau != 0.0f;
  if (open && pm_check(ctx, &tp->pm_open, n, arrs, 0, mem) != HSR_OK) return HSR_ERR_ARG;
  if (pm_check(ctx, &tp->pm_close, n, arrs, 0, mem) != HSR_OK) return HSR_ERR_ARG;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->tape = false;
  ctx->last_was_batch = false;
  ctx->tape_boxes = 0;
  cudaStream_t s = ctx->stream;
  const ArrayLayout A(n);
  float *f[8] = {x, y, z, vx, vy, vz, mass, phi};
  int64_t *ids = id;
  uint16_t *msk = mask;
  if (mem == HSR_MEM_HOST) {
    CU(ctx->d_res.ensure(A.bytes), "cudaMalloc(resident)");
    char *rb = ctx->d_res.as<char>();
    for (int i = 0; i < 8; ++i) {
      CU(cudaMemcpyAsync(rb + A.f[i], f[i], size_t(n) * 4, cudaMemcpyHostToDevice, s), "H2D arrays");
      f[i] = reinterpret_cast<float *>(rb + A.f[i]);
    }
    CU(cudaMemcpyAsync(rb + A.id, id, size_t(n) * 8, cudaMemcpyHostToDevice, s), "H2D ids");
    CU(cudaMemcpyAsync(rb + A.mask, mask, size_t(n) * 2, cudaMemcpyHostToDevice, s), "H2D masks");
    ids = reinterpret_cast<int64_t *>(rb + A.id);
    msk = reinterpret_cast<uint16_t *>(rb + A.mask);
  }
  hsr_pm_stats pm{};
  cudaEvent_t ev[4] = {ctx->ev0, ctx->ev1, ctx->ev2, ctx->ev3};
  std::string err;
  auto pm_kick = [&](const hsr_pm_params *pp) -> hsr_status {
    const hsr_pm::Params q = pm_params(pp);
    if (hsr_status r = pm_prepare(ctx, q)) return r;
    hsr_pm::Timing tm;
    if (!ctx->pm->kick(q, n, f[0], f[1], f[2], f[3], f[4], f[5], s, ev, &tm, &err))
      return ctx->fail(HSR_ERR_CUDA, err);
    pm.t_deposit_ms += tm.deposit_ms;
    pm.t_solve_ms += tm.solve_ms;
    pm.t_interp_ms += tm.interp_ms;
    pm.kernel_launches += tm.launches;
    pm.fft_execs += tm.fft_execs;
    return HSR_OK;
  };
  if (open)
    if (hsr_status r = pm_kick(&tp->pm_open)) return r;
  hsr_stats total{};
  int64_t inbox = n;
  if (hsr_status r = subcycle_resident(ctx, sp, n, f, ids, msk, &inbox, total)) return r;
  if (hsr_status r = pm_kick(&tp->pm_close)) return r;
  if (mem == HSR_MEM_HOST) {
    float *out[8] = {x, y, z, vx, vy, vz, mass, phi};
    for (int i = 0; i < 8; ++i)
      CU(cudaMemcpyAsync(out[i], f[i], size_t(n) * 4, cudaMemcpyDeviceToHost, s), "D2H arrays");
    CU(cudaMemcpyAsync(id, ids, size_t(n) * 8, cudaMemcpyDeviceToHost, s), "D2H ids");
    CU(cudaMemcpyAsync(mask, msk, size_t(n) * 2, cudaMemcpyDeviceToHost, s), "D2H masks");
    total.h2d_bytes = n * 42;
    total.d2h_bytes = n * 42;
  }
  CU(cudaStreamSynchronize(s), "TreePM step");
  if (n_inbox) *n_inbox = inbox;
  total.n = n;
  total.t_total_ms = ms_since(t_start);
  pm.t_total_ms = total.t_total_ms;
  ctx->stats = total;
  ctx->pm_stats = pm;
  ctx->have_lists = !sp->skip_kick && sp->nsub > 0;
  return HSR_OK;
}

hsr_status hsr_pm_vjp(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                      const float *y, const float *z, const float *vbx, const float *vby,
                      const float *vbz, float *xbx, float *xby, float *xbz, int32_t mem) {
  if (!ctx) return HSR_ERR_ARG;
  const auto t0 = clk::now();
  const void *arrs[9] = {x, y, z, vbx, vby, vbz, xbx, xby, xbz};
  hsr_status st = pm_check(ctx, p, n, arrs, 9, mem);
  if (st != HSR_OK) return st;
  CU(cudaSetDevice(ctx->device), "cudaSetDevice");
  const hsr_pm::Params q = pm_params(p);
  if ((st = pm_prepare(ctx, q)) != HSR_OK) return st;
  cudaStream_t s = ctx->stream;
  const float *in[6] = {x, y, z, vbx, vby, vbz};
  float *out[3] = {xbx, xby, xbz};
  const size_t nb = size_t(n) * sizeof(float);
  hsr_pm_stats ps{};
  if (mem == HSR_MEM_HOST && n > 0) {
    CU(ctx->d_pm.ensure(9 * nb), "cudaMalloc(PM adjoint)");
    float *b = ctx->d_pm.as<float>();
    for (int a = 0; a < 6; ++a) {
      CU(cudaMemcpyAsync(b + a * n, in[a], nb, cudaMemcpyHostToDevice, s), "PM adjoint copy in");
      in[a] = b + a * n;
    }
    for (int a = 0; a < 3; ++a) out[a] = b + (6 + a) * n;
    ps.h2d_bytes = int64_t(6 * nb);
    ps.d2h_bytes = int64_t(3 * nb);
  }
  const int64_t l0 = ctx->pm->launches, f0 = ctx->pm->fft_execs;
  std::string err;
  CU(cudaEventRecord(ctx->ev0, s), "event");
  if (!ctx->pm->vjp(q, n, in[0], in[1], in[2], in[3], in[4], in[5], out[0], out[1], out[2], s,
                    &err))
    return ctx->fail(HSR_ERR_CUDA, err);
  CU(cudaEventRecord(ctx->ev1, s), "event");
  if (mem == HSR_MEM_HOST && n > 0) {
    float *dst[3] = {xbx, xby, xbz};
    for (int a = 0; a < 3; ++a)
      CU(cudaMemcpyAsync(dst[a], out[a], nb, cudaMemcpyDeviceToHost, s), "PM adjoint copy out");
  }
  CU(cudaStreamSynchronize(s), "PM adjoint");
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ps.t_solve_ms = ms;  // the whole device part: deposits, four transforms, kernels
  ps.kernel_launches = ctx->pm->launches - l0;
  ps.fft_execs = ctx->pm->fft_execs - f0;
  ps.t_total_ms = ms_since(t0);
  ctx->pm_stats = ps;
  return HSR_OK;
}

hsr_status hsr_pm_get_stats(const hsr_ctx *ctx, hsr_pm_stats *st) {
  if (!ctx || !st) return HSR_ERR_ARG;
  *st = ctx->pm_stats;
  return HSR_OK;
}

}  // extern "C"
