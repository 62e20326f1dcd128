/*
 * RCBForceTree_gb300.h -- drop-in replacement for HACC's
 * src/halo_finder/RCBForceTree.h (class template RCBForceTree<TDPTS>,
 * RCBForceTree.h:92-203) that runs the short-range kick on a GB300 through the
 * C ABI in hacc_sr.h.
 *
 * Same constructor signature, argument meaning and in-place effect as the
 * reference (RCBForceTree.h:96-124, RCBForceTree.cxx:336-450): the constructor
 * builds the tree (permuting the ten particle arrays), builds the interaction
 * lists of the leaves inside the force box and kicks the velocities.  The
 * library implements one force law: the polynomial short-range law
 * (ForceLawSR over FGridEvalPoly, HACC's -P option) with softening `r`.
 * HACC selects that law only with -P; without it Particles builds ForceLawSR
 * over FGridEvalFit, and with -I over FGridEvalInterp
 * (src/cpu/Particles.cxx:173-183).  The constructor therefore evaluates
 * fl->f_over_r at a few separations and throws unless it is the polynomial
 * law at softening `r` (the Fit and Interp laws differ from it by 1e-4 to 1e-2
 * of the law's terms, rounding by 1e-7), so a run configured with another law
 * stops instead of silently changing the physics.  This needs the
 * reference's ForceLaw class, from the same "ForceLaw.h" the reference's
 * RCBForceTree.h includes.  Errors throw std::runtime_error where the
 * reference exits or asserts.  Each host thread uses its own context on
 * device HACC_SR_DEVICE (default 0), created on first use.
 */
#ifndef RCBFORCETREE_GB300_H
#define RCBFORCETREE_GB300_H

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "ForceLaw.h"  // the reference's ForceLaw (virtual float f_over_r(float r2))
#include "hacc_sr.h"

#define QUADRUPOLE_TDPTS 12
#define MONOPOLE_TDPTS 1

namespace hacc_sr_gb300 {

inline hsr_ctx *thread_context() {
  struct Holder {
    hsr_ctx *ctx = nullptr;
    ~Holder() {
      if (ctx) hsr_destroy(ctx);
    }
  };
  static thread_local Holder h;
  if (!h.ctx) {
    const char *dev = std::getenv("HACC_SR_DEVICE");
    hsr_status s = hsr_create(&h.ctx, dev ? std::atoi(dev) : 0);
    if (s != HSR_OK) throw std::runtime_error("hsr_create failed: status " + std::to_string(s));
  }
  return h.ctx;
}

// The law this library evaluates, in float as ForceLawSR::f_over_r computes
// it over FGridEvalPoly (src/halo_finder/ForceLaw.cxx:98-104, 187-192):
// powf(r2 + rsm2, -1.5) - sum_k a_k r2^k.  *scale receives the size of the
// two terms, the yardstick of the comparison below.
inline float poly6_law(float r2, float rsm2, float *scale = nullptr) {
  const float a[7] = {0.271431f,    -0.0783394f,      0.0133122f,     -0.00159485f,
                      0.000132336f, -0.00000663394f, 0.000000147305f};
  const float p = a[0] + r2 * (a[1] + r2 * (a[2] + r2 * (a[3] + r2 * (a[4] + r2 * (a[5] + r2 * a[6])))));
  const float y = std::pow(r2 + rsm2, -1.5f);
  if (scale) *scale = std::fabs(y) + std::fabs(p);
  return y - p;
}

// Throws unless fl->f_over_r is the polynomial law at softening rsm: at
// separations r2 from 0.05 to 9 (inside the cutoff, 3.116^2) the two must
// agree within 4e-6 of the law's terms.  The Fit law misses by 12 to 40 times
// that at every one of these points, a wrong softening by far more.
inline void require_poly6_law(ForceLaw *fl, float rsm, const char *who) {
  const float r2s[8] = {0.05f, 0.3f, 1.0f, 2.0f, 4.0f, 6.5f, 9.0f, 9.6f};
  for (float r2 : r2s) {
    float scale = 0.f;
    const float want = poly6_law(r2, rsm * rsm, &scale);
    const float got = fl->f_over_r(r2);
    if (!(std::fabs(got - want) <= 4e-6f * scale))
      throw std::runtime_error(
          std::string(who) + ": the ForceLaw is not the polynomial short-range law "
          "(ForceLawSR over FGridEvalPoly, HACC option -P) at softening " + std::to_string(rsm) +
          " -- f_over_r(" + std::to_string(r2) + ") = " + std::to_string(got) + ", expected " +
          std::to_string(want) + "; this library implements that law only");
  }
}

// The softening of a polynomial short-range law, read off the law itself:
// f_over_r(0) = rsm^-3 - a_0.  Of the floats next to the closed-form value the
// one whose law reproduces f_over_r(0) exactly is taken; -1 when none is
// positive and finite.
inline float law_softening(ForceLaw *fl) {
  const float g0 = fl->f_over_r(0.0f);
  const float t = g0 + 0.271431f;
  if (!(t > 0.f) || !std::isfinite(t)) return -1.f;
  const float c = std::pow(t, -1.0f / 3.0f);
  float cand[5] = {c, std::nextafter(c, 0.f), std::nextafter(c, INFINITY), 0.f, 0.f};
  cand[3] = std::nextafter(cand[1], 0.f);
  cand[4] = std::nextafter(cand[2], INFINITY);
  for (float r : cand)
    if (poly6_law(0.f, r * r) == g0) return r;
  return c;
}

}  // namespace hacc_sr_gb300

template <int TDPTS>
class RCBForceTree {
 public:
  RCBForceTree(float *minLoc, float *maxLoc, float *minForceLoc, float *maxForceLoc,
               int64_t count, float *xLoc, float *yLoc, float *zLoc, float *xVel, float *yVel,
               float *zVel, float *mass, float *phiLoc, int64_t *idLoc, uint16_t *maskLoc,
               float avgMass, float fsm, float r, float oa, int64_t nd = 1, int64_t ds = 1,
               int64_t tmin = 128, ForceLaw *fl = 0, float fcoeff = 0.0, float ppc = 0.9) {
    if (!fl)
      throw std::runtime_error(
          "RCBForceTree (GB300): fl == 0 selects the Newtonian law, which is not the "
          "short-range path this library implements");
    hacc_sr_gb300::require_poly6_law(fl, r, "RCBForceTree (GB300)");
    hsr_params p{};
    for (int i = 0; i < 3; ++i) {
      p.min[i] = minLoc[i];
      p.max[i] = maxLoc[i];
      p.min_force[i] = minForceLoc[i];
      p.max_force[i] = maxForceLoc[i];
    }
    p.avg_mass = avgMass;
    p.fsrrmax = fsm;
    p.rsm = r;
    p.open_angle = oa;
    p.nd = nd;
    p.ds = ds;
    p.tmin = tmin;
    p.fcoeff = fcoeff;
    p.ppc = ppc;
    p.tdpts = TDPTS;
    p.law = HSR_LAW_POLY6;
    p.kernel = HSR_KERNEL_AUTO;
    hsr_ctx *ctx = hacc_sr_gb300::thread_context();
    hsr_status s = hsr_rcb_kick(ctx, &p, count, xLoc, yLoc, zLoc, xVel, yVel, zVel, mass, phiLoc,
                                idLoc, maskLoc, HSR_MEM_HOST);
    if (s != HSR_OK)
      throw std::runtime_error(std::string("hsr_rcb_kick: ") + hsr_last_error(ctx));
    hsr_get_stats(ctx, &stats_);
  }

  ~RCBForceTree() {}

  // printStats (RCBForceTree.cxx:461-511) equivalent: the call's statistics.
  const hsr_stats &stats() const { return stats_; }

 private:
  hsr_stats stats_{};
};

typedef RCBForceTree<QUADRUPOLE_TDPTS> RCBQuadrupoleForceTree;
typedef RCBForceTree<MONOPOLE_TDPTS> RCBMonopoleForceTree;

#endif /* RCBFORCETREE_GB300_H */
