// rcb_host.cpp -- RCB tree build and interaction lists on the host.
//
// Compiled with -ffp-contract=off: every float expression that decides the
// tree or a list (centre of mass, split, opening test, pseudo-particles) must
// round exactly as the reference's does, and the reference never fuses a
// multiply with an add on x86-64.
#include "rcb_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace hsr {

// ---------------------------------------------------------------------------
// Pool
// ---------------------------------------------------------------------------

Pool::Pool(int nthreads) : nthreads_(std::max(1, nthreads)) {
  for (int i = 1; i < nthreads_; ++i) threads_.emplace_back([this, i] { worker(i); });
}

Pool::~Pool() {
  {
    std::lock_guard<std::mutex> g(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  for (auto &t : threads_) t.join();
}

void Pool::run_chunks() {
  for (;;) {
    int64_t b = next_.fetch_add(job_grain_);
    if (b >= job_n_) break;
    (*job_)(b, std::min(b + job_grain_, job_n_));
  }
}

void Pool::worker(int) {
  uint64_t seen = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
    }
    run_chunks();
    {
      std::lock_guard<std::mutex> g(mu_);
      if (--pending_ == 0) done_cv_.notify_all();
    }
  }
}

void Pool::parallel_for(int64_t n, int64_t grain,
                        const std::function<void(int64_t, int64_t)> &fn) {
  if (n <= 0) return;
  grain = std::max<int64_t>(1, grain);
  if (nthreads_ == 1 || n <= grain) {
    fn(0, n);
    return;
  }
  {
    std::lock_guard<std::mutex> g(mu_);
    job_ = &fn;
    job_n_ = n;
    job_grain_ = grain;
    next_.store(0);
    pending_ = nthreads_ - 1;
    ++gen_;
  }
  cv_.notify_all();
  run_chunks();
  std::unique_lock<std::mutex> lk(mu_);
  done_cv_.wait(lk, [&] { return pending_ == 0; });
  job_ = nullptr;
}

// ---------------------------------------------------------------------------
// Geometry helpers (RCBForceTree.cxx:519-569)
// ---------------------------------------------------------------------------

namespace {

// Unit design points: the centre of mass for one pseudo-particle
// (RCBForceTree.cxx:134-144) and the 12 icosahedron vertices of Hardin and
// Sloane in the reference's order (RCBForceTree.cxx:227-272).
constexpr float kIcoA = 0.525731112119134f;
constexpr float kIcoB = 0.85065080835204f;
const float kIco[12][3] = {
    {0, kIcoB, kIcoA},   {0, kIcoB, -kIcoA},  {kIcoA, 0, kIcoB},   {-kIcoA, 0, kIcoB},
    {kIcoB, kIcoA, 0},   {-kIcoB, kIcoA, 0},  {0, -kIcoB, -kIcoA}, {0, -kIcoB, kIcoA},
    {-kIcoA, 0, -kIcoB}, {kIcoA, 0, -kIcoB},  {-kIcoB, -kIcoA, 0}, {kIcoB, -kIcoA, 0}};
const float kMono[1][3] = {{0, 0, 0}};

inline const float (*design(int k))[3] { return k == 12 ? kIco : kMono; }

// std::min semantics: (b < a) ? b : a.
inline float smin(float a, float b) { return (b < a) ? b : a; }

inline float pptdr(const Node &t) {
  return smin(t.xmax[0] - t.xc[0],
              smin(t.xmax[1] - t.xc[1],
                   smin(t.xmax[2] - t.xc[2],
                        smin(t.xc[0] - t.xmin[0], smin(t.xc[1] - t.xmin[1], t.xc[2] - t.xmin[2])))));
}

inline void pppts(int k, float tdr, const float *xc, float *px, float *py, float *pz) {
  const float(*d)[3] = design(k);
  for (int i = 0; i < k; ++i) {
    px[i] = tdr * d[i][0] + xc[0];
    py[i] = tdr * d[i][1] + xc[1];
    pz[i] = tdr * d[i][2] + xc[2];
  }
}

// Pseudo-particle mass accumulation over `count` sources (x, y, z, m given by
// accessors), matching the monopole, dipole and quadrupole moments.
template <typename Src>
void pp_accum(int k, int64_t count, Src src, const float *xc, const float *px,
              const float *py, const float *pz, float *ppm, float tdr) {
  const float K = float(k);
  const float odr0 = 1 / K;
  for (int i = 0; i < count; ++i) {
    float sx, sy, sz, sm;
    src(i, sx, sy, sz, sm);
    float xi = sx - xc[0];
    float yi = sy - xc[1];
    float zi = sz - xc[2];
    float ri = std::sqrt(xi * xi + yi * yi + zi * zi);
    for (int j = 0; j < k; ++j) {
      float xj = px[j] - xc[0];
      float yj = py[j] - xc[1];
      float zj = pz[j] - xc[2];
      float rj2 = xj * xj + yj * yj + zj * zj;
      float odr1 = 0, odr2 = 0;
      if (rj2 != 0) {
        float rj = std::sqrt(rj2);
        float aij = (xi * xj + yi * yj + zi * zj) / (ri * rj);
        odr1 = (3 / K) * (ri / tdr) * aij;
        odr2 = float(double((5 / K) * (ri / tdr) * (ri / tdr)) * 0.5 * double(3 * aij * aij - 1));
      }
      ppm[j] += sm * (odr0 + odr1 + odr2);
    }
  }
}

// fminf / fmaxf of the reference's cm (BGQCM.c:193-198) without the libm
// call: the non-NaN operand where one is NaN, else the smaller (larger).
// Where both operands are zeros of either sign the result may carry the other
// sign than libm's; no split, opening test or sum depends on the sign of a
// zero bound (they take differences and comparisons of the bounds only).
inline float bound_min(float a, float b) { return (b < a || a != a) ? b : a; }
inline float bound_max(float a, float b) { return (b > a || a != a) ? b : a; }

}  // namespace

// ---------------------------------------------------------------------------
// Build
// ---------------------------------------------------------------------------

RcbHost::RcbHost(int nthreads) : pool_(nthreads) {}

int32_t RcbHost::alloc_nodes(int k) {
  std::lock_guard<std::mutex> g(alloc_mu_);
  int64_t i = num_alloc_.load();
  num_alloc_.store(i + k);
  for (int64_t j = i; j < i + k; ++j) {
    auto &c = chunks_[j >> kChunkBits];
    if (!c) c.reset(new Node[kChunk]);
    N(j) = Node();
  }
  return int32_t(i);
}

// Bounding box and centre of mass, in array order with double sums
// (BGQCM.c:181-212; RCOForceTree.cxx's cm is the same).
void RcbHost::node_stats(Node &T) {
  const int64_t cnt = T.count;
  const Elem *e = elems_.data() + T.offset;
  double sx = 0, sy = 0, sz = 0, sm = 0;
  if (cnt > 0) {
    // the bounds stay in registers (as far as the compiler knows, the node
    // could alias the elements)
    float x0 = e[0].x, x1 = e[0].x, y0 = e[0].y, y1 = e[0].y, z0 = e[0].z, z1 = e[0].z;
    for (int64_t i = 0; i < cnt; ++i) {
      const Elem &q = e[i];
      x0 = bound_min(x0, q.x);
      x1 = bound_max(x1, q.x);
      y0 = bound_min(y0, q.y);
      y1 = bound_max(y1, q.y);
      z0 = bound_min(z0, q.z);
      z1 = bound_max(z1, q.z);
      const float w = q.m;
      sx += double(w * q.x);
      sy += double(w * q.y);
      sz += double(w * q.z);
      sm += double(w);
    }
    T.xmin[0] = x0;
    T.xmax[0] = x1;
    T.xmin[1] = y0;
    T.xmax[1] = y1;
    T.xmin[2] = z0;
    T.xmax[2] = z1;
  }
  T.xc[0] = float(sx / sm);
  T.xc[1] = float(sy / sm);
  T.xc[2] = float(sz / sm);
}

// Pseudo-particles of a leaf from its own particles (RCBForceTree.cxx:788-800).
void RcbHost::leaf_pseudo(Node &T) {
  const int k = p_.tdpts;
  const Elem *e = elems_.data() + T.offset;
  T.tdr = p_.ppc * pptdr(T);
  std::fill(T.ppm, T.ppm + 12, 0.0f);
  if (T.count > k) {
    float px[12], py[12], pz[12];
    pppts(k, T.tdr, T.xc, px, py, pz);
    auto own = [e](int64_t i, float &x, float &y, float &z, float &m) {
      x = e[i].x; y = e[i].y; z = e[i].z; m = e[i].m;
    };
    pp_accum(k, T.count, own, T.xc, px, py, pz, T.ppm, T.tdr);
  }
}

// Pseudo-particles of an inner node from its children, in child order
// (RCBForceTree.cxx:856-889; RCOForceTree.cxx:716-737).
void RcbHost::pseudo_from_children(Node &T, const int32_t *kids, int nk) {
  const int k = p_.tdpts;
  float px[12], py[12], pz[12];
  T.tdr = p_.ppc * pptdr(T);
  pppts(k, T.tdr, T.xc, px, py, pz);
  std::fill(T.ppm, T.ppm + 12, 0.0f);
  for (int j = 0; j < nk; ++j) {
    const Node *C = &N(kids[j]);
    if (C->count <= 0) continue;
    if (C->count <= k) {
      const Elem *ce = elems_.data() + C->offset;
      auto src = [ce](int64_t i, float &x, float &y, float &z, float &m) {
        x = ce[i].x; y = ce[i].y; z = ce[i].z; m = ce[i].m;
      };
      pp_accum(k, C->count, src, T.xc, px, py, pz, T.ppm, T.tdr);
    } else {
      float cx[12], cy[12], cz[12];
      pppts(k, C->tdr, C->xc, cx, cy, cz);
      const float *cm = C->ppm;
      auto src = [&](int64_t i, float &x, float &y, float &z, float &m) {
        x = cx[i]; y = cy[i]; z = cz[i]; m = cm[i];
      };
      pp_accum(k, k, src, T.xc, px, py, pz, T.ppm, T.tdr);
    }
  }
}

void RcbHost::build_node(int32_t tl, int depth) {
  Node &T = N(tl);
  const int64_t cnt = T.count, off = T.offset;
  Elem *e = elems_.data() + off;
  node_stats(T);
  if (cnt <= p_.nd) {  // leaf (RCBForceTree.cxx:788-800)
    leaf_pseudo(T);
    return;
  }

  const int32_t tlcl = alloc_nodes(2), tlcr = tlcl + 1;
  Node &L = N(tlcl), &R = N(tlcr);
  for (int i = 0; i < 3; ++i) {
    L.xmin[i] = R.xmin[i] = T.xmin[i];
    L.xmax[i] = R.xmax[i] = T.xmax[i];
  }
  float xlen[3];
  for (int i = 0; i < 3; ++i) xlen[i] = T.xmax[i] - T.xmin[i];
  int d;
  if (xlen[0] > xlen[1] && xlen[0] > xlen[2]) d = 0;
  else if (xlen[1] > xlen[2]) d = 1;
  else d = 2;

  // Partition at the centre of mass (RCBForceTree.cxx:623-672, 719-729):
  // the indices below the split are collected in order and the j-th of them
  // is swapped into slot j.
  const float split = T.xc[d];
  static thread_local std::vector<int32_t> idx;
  if (int64_t(idx.size()) < cnt) idx.resize(size_t(cnt));
  int64_t is = 0;
  if (d == 0) {
    for (int64_t i = 0; i < cnt; ++i) if (e[i].x < split) idx[is++] = int32_t(i);
  } else if (d == 1) {
    for (int64_t i = 0; i < cnt; ++i) if (e[i].y < split) idx[is++] = int32_t(i);
  } else {
    for (int64_t i = 0; i < cnt; ++i) if (e[i].z < split) idx[is++] = int32_t(i);
  }
  for (int64_t j = 0; j < is; ++j) std::swap(e[idx[j]], e[j]);

  if (is != 0 && is != cnt) {
    L.count = is;
    R.count = cnt - is;
    T.c[0] = tlcl;
    L.offset = off;
    L.xmax[d] = split;
    T.c[1] = tlcr;
    R.offset = off + is;
    R.xmin[d] = split;
    if (depth < par_depth_) {
      std::thread th([this, tlcl, depth] { build_node(tlcl, depth + 1); });
      build_node(tlcr, depth + 1);
      th.join();
    } else {
      build_node(tlcl, depth + 1);
      build_node(tlcr, depth + 1);
    }
  }
  const int32_t kids[2] = {tlcl, tlcr};
  pseudo_from_children(T, kids, 2);
}

// The RCO octree (RCOForceTree.cxx:580-738): every inner node splits all three
// axes at its centre of mass into up to eight children.  Partition, in one
// pass in array order: a particle of octant p < 7 (coordinates at or above
// the split add 4, 2, 1 for x, y, z) moves to the end of octant p's run, and
// the first particle of each later run moves to that run's end in turn; the
// particles of octant 7 stay behind the runs.  (The reference's swap chain
// starts from is[7] of a 7-entry array; the end of the processed range, i,
// is the value the chain needs there.)
void RcbHost::build_node_oct(int32_t tl, int depth) {
  Node &T = N(tl);
  const int64_t cnt = T.count, off = T.offset;
  Elem *e = elems_.data() + off;
  node_stats(T);
  if (cnt <= p_.nd) {
    leaf_pseudo(T);
    return;
  }
  const int32_t c0 = alloc_nodes(8);
  for (int j = 0; j < 8; ++j) {
    Node &C = N(c0 + j);
    for (int i = 0; i < 3; ++i) {
      C.xmin[i] = T.xmin[i];
      C.xmax[i] = T.xmax[i];
    }
  }
  const float sx = T.xc[0], sy = T.xc[1], sz = T.xc[2];
  int64_t is[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = 0; i < cnt; ++i) {
    const int p = (e[i].x >= sx ? 4 : 0) + (e[i].y >= sy ? 2 : 0) + (e[i].z >= sz ? 1 : 0);
    if (p == 7) continue;
    is[7] = i;
    std::swap(e[is[7]], e[i]);
    for (int q = 7; q > p; --q) std::swap(e[is[q - 1]], e[is[q]]);
    for (int q = p; q < 7; ++q) ++is[q];
  }
  bool div = false;
  for (int q = 0; q < 7; ++q) div |= !(is[q] == 0 || is[q] == cnt);
  int32_t kids[8];
  for (int j = 0; j < 8; ++j) kids[j] = c0 + j;
  if (div) {
    int64_t counts[8];
    counts[0] = is[0];
    for (int q = 1; q < 7; ++q) counts[q] = is[q] - is[q - 1];
    counts[7] = cnt - is[6];
    int64_t coff = off;
    std::vector<std::thread> ths;
    for (int j = 0; j < 8; ++j) {
      Node &C = N(c0 + j);
      C.count = counts[j];
      if (counts[j] <= 0) continue;
      T.c[j] = c0 + j;
      C.offset = coff;
      coff += counts[j];
    }
    for (int j = 0; j < 8; ++j) {
      if (T.c[j] <= 0) continue;
      if (depth < par_depth_oct_) ths.emplace_back([this, c0, j, depth] { build_node_oct(c0 + j, depth + 1); });
      else build_node_oct(c0 + j, depth + 1);
    }
    for (auto &th : ths) th.join();
  }
  pseudo_from_children(T, kids, 8);
}

void RcbHost::build(const TreeParams &p, int64_t n, const float *x, const float *y,
                    const float *z, const float *m) {
  p_ = p;
  n_ = n;
  elems_.resize(size_t(n));
  pool_.parallel_for(n, 1 << 16, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) elems_[i] = Elem{x[i], y[i], z[i], m[i], int32_t(i)};
  });
  chunks_.clear();
  chunks_.resize(size_t((((p.tree == 1 ? 8 : 2) * n + 9) >> kChunkBits) + 2));
  num_alloc_.store(1);
  chunks_[0].reset(new Node[kChunk]);
  N(0) = Node();
  Node &root = N(0);
  root.count = n;
  root.offset = 0;
  for (int i = 0; i < 3; ++i) {
    root.xmin[i] = p.min[i];
    root.xmax[i] = p.max[i];
  }
  par_depth_ = 0;
  while ((1 << par_depth_) < 2 * pool_.size()) ++par_depth_;
  par_depth_oct_ = 0;
  while ((1 << (3 * par_depth_oct_)) < 2 * pool_.size()) ++par_depth_oct_;
  if (p.tree == 1) build_node_oct(0, 0);
  else build_node(0, 0);

  num_nodes_ = num_alloc_.load();
  flat_.resize(size_t(num_nodes_));
  pool_.parallel_for(num_nodes_, 1 << 14, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) flat_[i] = N(i);
  });
  chunks_.clear();
}

void RcbHost::pseudo_table(float *out) const {
  const int k = p_.tdpts;
  const_cast<Pool &>(pool_).parallel_for(num_nodes_, 4096, [&](int64_t b, int64_t e) {
    for (int64_t t = b; t < e; ++t) {
      const Node &T = flat_[t];
      float px[12], py[12], pz[12];
      pppts(k, T.tdr, T.xc, px, py, pz);
      for (int i = 0; i < k; ++i) {
        float *o = out + 4 * (t * k + i);
        o[0] = px[i];
        o[1] = py[i];
        o[2] = pz[i];
        o[3] = T.ppm[i];
      }
    }
  });
}

int64_t RcbHost::padded_pairs() const {
  int64_t s = 0;
  for (const auto &L : leaves_) s += ((L.count + 31) / 32) * 32 * L.list_len;
  return s;
}

int64_t RcbHost::nonempty_leaves() const {
  int64_t c = 0;
  for (int64_t t = 1; t < num_nodes_; ++t)
    if (flat_[t].leaf() && flat_[t].count > 0) ++c;
  return c;
}

// ---------------------------------------------------------------------------
// Interaction lists (RCBForceTree.cxx:923-1197)
// ---------------------------------------------------------------------------

void RcbHost::leaf_list(int64_t tl, std::vector<Seg> &out, std::vector<int32_t> &st) const {
  const Node &T = flat_[tl];
  const float fsr = p_.fsrrmax;
  const float fsr2 = fsr * fsr;
  const float tan_oa = p_.tan_oa;
  const int k = p_.tdpts;
  auto emit = [&](int64_t start, int64_t count) {
    if (count > 0) out.push_back(Seg{int32_t(start), int32_t(count)});
  };
  // Per-axis gap between the target leaf's box and a child's box.
  auto close = [&](const Node &C) {
    for (int i = 0; i < 3; ++i) {
      float dist = 0;
      if (T.xmax[i] < C.xmin[i]) dist = C.xmin[i] - T.xmax[i];
      else if (T.xmin[i] > C.xmax[i]) dist = T.xmin[i] - C.xmax[i];
      if (dist > fsr) return false;
    }
    return true;
  };

  st.clear();
  st.push_back(0);
  while (!st.empty()) {
    const int32_t t = st.back();
    st.pop_back();
    const Node &Q = flat_[t];

    // Ancestors of the target: descend without interacting.  Tree ranges are
    // nested or disjoint, so containment of the target's range identifies them.
    if (t != tl && Q.offset <= T.offset && T.offset + T.count <= Q.offset + Q.count) {
      for (int j = 0; j < 8; ++j) {
        const int32_t c = Q.c[j];
        if (c != tl && c > 0 && flat_[c].count > 0) st.push_back(c);
      }
      continue;
    }

    const float dx = Q.xc[0] - T.xc[0];
    const float dy = Q.xc[1] - T.xc[1];
    const float dz = Q.xc[2] - T.xc[2];
    const float dist2 = dx * dx + dy * dy + dz * dz;
    const float sx = Q.xmax[0] - Q.xmin[0];
    const float sy = Q.xmax[1] - Q.xmin[1];
    const float sz = Q.xmax[2] - Q.xmin[2];
    const float l2 = smin(sx * sx, smin(sy * sy, sz * sz));
    const float dtt2 = dist2 * tan_oa * tan_oa;
    bool big = l2 > dtt2;
    for (int i = 0; i < 2 && !big; ++i)
      for (int j = 0; j < 2 && !big; ++j) {
        const float x1 = (i == 0 ? Q.xmin : Q.xmax)[0] - T.xc[0];
        const float y1 = (j == 0 ? Q.xmin : Q.xmax)[1] - T.xc[1];
        const float z1 = Q.xmin[2] - T.xc[2];
        const float x2 = (i == 0 ? Q.xmax : Q.xmin)[0] - T.xc[0];
        const float y2 = (j == 0 ? Q.xmax : Q.xmin)[1] - T.xc[1];
        const float z2 = Q.xmax[2] - T.xc[2];
        const float ddx = x1 - x2, ddy = y1 - y2, ddz = z1 - z2;
        const float dh2 = ddx * ddx + ddy * ddy + ddz * ddz;
        big = dh2 > dtt2;
      }

    if (!big) {
      if (dist2 > fsr2) continue;  // too far to matter, children included
      if (Q.count <= k) emit(Q.offset, Q.count);
      else emit(n_ + int64_t(t) * k, k);
      continue;
    }
    if (Q.leaf()) {
      emit(Q.offset, Q.count);
      continue;
    }
    for (int j = 0; j < 8; ++j) {
      const int32_t c = Q.c[j];
      if (c > 0 && flat_[c].count > 0 && close(flat_[c])) st.push_back(c);
    }
  }
  emit(T.offset, T.count);  // self interactions last
}

void RcbHost::walk() {
  // Leaves inside the force box, in the reference's DFS order.
  std::vector<int32_t> lv;
  {
    std::vector<int32_t> q{0};
    std::vector<int32_t> parents;
    while (!q.empty()) {
      const int32_t tl = q.back();
      const Node &T = flat_[tl];
      if (T.leaf()) {
        q.pop_back();
        bool inside = true;
        for (int i = 0; i < 3; ++i)
          inside &= (T.xmax[i] < p_.max_force[i] && T.xmax[i] > p_.min_force[i]) ||
                    (T.xmin[i] < p_.max_force[i] && T.xmin[i] > p_.min_force[i]);
        if (inside) lv.push_back(tl);
      } else if (!parents.empty() && parents.back() == tl) {
        parents.pop_back();
        q.pop_back();
      } else {
        for (int j = 0; j < 8; ++j)
          if (T.c[j] > 0) q.push_back(T.c[j]);
        parents.push_back(tl);
      }
    }
  }

  const int64_t nl = int64_t(lv.size());
  const int64_t grain = 8;
  const int64_t nchunks = (nl + grain - 1) / grain;
  std::vector<std::vector<Seg>> chunk_segs(static_cast<size_t>(nchunks));
  leaves_.assign(size_t(nl), LeafWork{});
  pool_.parallel_for(nchunks, 1, [&](int64_t cb, int64_t ce) {
    std::vector<int32_t> stack;
    stack.reserve(256);
    for (int64_t c = cb; c < ce; ++c) {
      auto &out = chunk_segs[c];
      for (int64_t l = c * grain; l < std::min(nl, (c + 1) * grain); ++l) {
        const size_t b = out.size();
        leaf_list(lv[l], out, stack);
        int64_t len = 0;
        for (size_t s = b; s < out.size(); ++s) len += out[s].count;
        const Node &T = flat_[lv[l]];
        leaves_[l] = LeafWork{T.offset, T.count, int64_t(b), int64_t(out.size()), len};
      }
    }
  });
  // Concatenate the chunks in leaf order.
  std::vector<int64_t> base(size_t(nchunks) + 1, 0);
  for (int64_t c = 0; c < nchunks; ++c) base[c + 1] = base[c] + int64_t(chunk_segs[c].size());
  segs_.resize(size_t(base[nchunks]));
  pool_.parallel_for(nchunks, 4, [&](int64_t cb, int64_t ce) {
    for (int64_t c = cb; c < ce; ++c) {
      std::copy(chunk_segs[c].begin(), chunk_segs[c].end(), segs_.begin() + base[c]);
      for (int64_t l = c * grain; l < std::min(nl, (c + 1) * grain); ++l) {
        leaves_[l].seg_begin += base[c];
        leaves_[l].seg_end += base[c];
      }
    }
  });
  list_entries_ = 0;
  pairs_ = 0;
  for (const auto &L : leaves_) {
    list_entries_ += L.list_len;
    pairs_ += L.count * L.list_len;
  }
}

}  // namespace hsr
