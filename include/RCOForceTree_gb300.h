/*
 * RCOForceTree_gb300.h -- drop-in replacement for HACC's
 * src/halo_finder/RCOForceTree.h (class template RCOForceTree<TDPTS>, the
 * octree variant selected by HACC's -O option, src/cpu/Particles.cxx:
 * 1259-1310) that runs the short-range kick through the C ABI in hacc_sr.h.
 *
 * Same constructor signature and in-place effect as the reference
 * (RCOForceTree.h:95-121, RCOForceTree.cxx:326-412): the octree is built on
 * the host (every inner node split along all three axes at its centre of
 * mass, the ten particle arrays permuted), the lists of the leaves inside the
 * force box are built there, and the pairs run on the GPU.  The reference
 * takes the softening from its ForceLaw object (the constructor has no rsm
 * argument); this header reads it off the law, f_over_r(0) = rsm^-3 - a_0,
 * and then checks the law as RCBForceTree_gb300.h does: anything but the
 * polynomial short-range law (HACC option -P) throws.
 */
#ifndef RCOFORCETREE_GB300_H
#define RCOFORCETREE_GB300_H

#include "RCBForceTree_gb300.h"

template <int TDPTS>
class RCOForceTree {
 public:
  RCOForceTree(float *minLoc, float *maxLoc, float *minForceLoc, float *maxForceLoc,
               int64_t count, float *xLoc, float *yLoc, float *zLoc, float *xVel, float *yVel,
               float *zVel, float *mass, float *phiLoc, int64_t *idLoc, uint16_t *maskLoc,
               float avgMass, float fsm, float oa, int64_t nd = 1, int64_t ds = 1,
               ForceLaw *fl = 0, float fcoeff = 0.0, float ppc = 0.9) {
    if (!fl)
      throw std::runtime_error(
          "RCOForceTree (GB300): fl == 0 selects the Newtonian law, which is not the "
          "short-range path this library implements");
    const float rsm = hacc_sr_gb300::law_softening(fl);
    if (!(rsm > 0.f))
      throw std::runtime_error(
          "RCOForceTree (GB300): the ForceLaw has no finite softening at r2 = 0; this library "
          "implements the polynomial short-range law (ForceLawSR over FGridEvalPoly) only");
    hacc_sr_gb300::require_poly6_law(fl, rsm, "RCOForceTree (GB300)");
    hsr_params p{};
    for (int i = 0; i < 3; ++i) {
      p.min[i] = minLoc[i];
      p.max[i] = maxLoc[i];
      p.min_force[i] = minForceLoc[i];
      p.max_force[i] = maxForceLoc[i];
    }
    p.avg_mass = avgMass;
    p.fsrrmax = fsm;
    p.rsm = rsm;
    p.open_angle = oa;
    p.nd = nd;
    p.ds = ds;
    p.fcoeff = fcoeff;
    p.ppc = ppc;
    p.tdpts = TDPTS;
    p.law = HSR_LAW_POLY6;
    p.kernel = HSR_KERNEL_AUTO;
    p.tree = HSR_TREE_RCO;
    hsr_ctx *ctx = hacc_sr_gb300::thread_context();
    hsr_status s = hsr_rcb_kick(ctx, &p, count, xLoc, yLoc, zLoc, xVel, yVel, zVel, mass, phiLoc,
                                idLoc, maskLoc, HSR_MEM_HOST);
    if (s != HSR_OK)
      throw std::runtime_error(std::string("hsr_rcb_kick (RCO): ") + hsr_last_error(ctx));
    hsr_get_stats(ctx, &stats_);
  }

  ~RCOForceTree() {}

  const hsr_stats &stats() const { return stats_; }

 private:
  hsr_stats stats_{};
};

typedef RCOForceTree<QUADRUPOLE_TDPTS> RCOQuadrupoleForceTree;
typedef RCOForceTree<MONOPOLE_TDPTS> RCOMonopoleForceTree;

#endif /* RCOFORCETREE_GB300_H */
