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
 * force law is the polynomial short-range law (ForceLawSR over FGridEvalPoly,
 * HACC's -P option) with softening `r`; Particles::map2 passes the same m_rsm
 * as `r` and to its ForceLawSR (src/cpu/Particles.cxx:1313-1336), so `fl` is
 * only checked for null.  Errors throw std::runtime_error where the reference
 * exits or asserts.  Each host thread uses its own context on device
 * HACC_SR_DEVICE (default 0), created on first use.
 */
#ifndef RCBFORCETREE_GB300_H
#define RCBFORCETREE_GB300_H

#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "hacc_sr.h"

class ForceLaw;  // the reference's force-law base class (only its pointer is used)

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
          "short-range path this build implements");
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
