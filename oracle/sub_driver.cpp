// sub_driver.cpp -- runs the reference's own short-range sub-cycle,
// Particles::subCycle (src/cpu/Particles.cxx:1176-1201: map1, map2 with
// resortParticles and the RCB force tree, map1), with the reference's
// TimeStepper (src/simulation/TimeStepper.cxx), all compiled unmodified from
// the reference sources by oracle/Makefile (target _ref/sub_ref).
//
// TEST INFRASTRUCTURE ONLY: used to pin the CPU restatement of the sub-cycle
// (ora_map1, ora_resort and the kick coefficient) and of the time stepper.
// Never part of the product.
//
// Usage: sub_ref <sub.bin> <out.bin>
// Input: 8-byte magic "HSRSUBC1", int64 n, the SubParams block, the ten
// particle arrays (x, y, z, vx, vy, vz, mass, phi as float; id int64; mask
// uint16).  The driver builds the TimeStepper (alpha, ain, afin, nsteps,
// omegatot), advances it half_steps half steps, runs subCycle on the arrays
// (a Particles object whose members are set directly: its constructor reads
// an input deck and initialises MPI), writes the arrays back in the same
// format and prints one JSON line with the stepper's values and m_Np_last.

// the standard headers first: only the reference's own classes see the
// access change below
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <new>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define private public  // Particles' and Domain's members are set directly
#include "Particles.h"
#undef private

// Storage for the Partition statics the force tree reads (rank number only).
int Partition::myProc = 0;
int Partition::numProc = 1;

namespace {

struct SubParams {
  double alpha, ain, afin, omegatot;      // TimeStepper(alpha, ain, afin, nsteps, omegatot)
  int64_t ppn, extra_levels, task_part_min;  // m_rcbTreePPN, ...ExtraLevels, ...TaskPartMin
  int32_t ng[3];                          // Domain::ng_local_total
  int32_t nsub, nsteps, half_steps;       // sub-cycles; stepper steps; half steps advanced
  int32_t use_rcb_tree;                   // m_useRCBTree: 2 RCB mono, 1 RCB quad, 5 RCO mono, 4 RCO quad
  int32_t skip_stream, skip_kick, nthreads;
  float edge, gpscal, rsm, open_angle;    // m_edge, m_gpscal, m_rsm, m_openAngle
};

template <typename T>
bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <typename T>
bool wr(FILE *f, const T *p, size_t n) { return fwrite(p, sizeof(T), n, f) == n; }

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s sub.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror("open input"); return 2; }
  char magic[8];
  int64_t n = 0;
  SubParams S;
  if (!rd(f, magic, 8) || memcmp(magic, "HSRSUBC1", 8) != 0 || !rd(f, &n, 1) || !rd(f, &S, 1)) {
    fprintf(stderr, "bad input file\n");
    return 2;
  }
  // 64-byte aligned arrays, as Particles allocates them
  auto falloc = [](int64_t m) {
    void *p = nullptr;
    if (posix_memalign(&p, 64, size_t(m > 0 ? m : 1) * sizeof(float))) return (float *)nullptr;
    return (float *)p;
  };
  float *a[8];
  for (auto &v : a) {
    v = falloc(n);
    if (!v || (n && !rd(f, v, n))) return 2;
  }
  std::vector<int64_t> id(n);
  std::vector<uint16_t> mask(n);
  if (n && (!rd(f, id.data(), n) || !rd(f, mask.data(), n))) return 2;
  fclose(f);
#ifdef _OPENMP
  if (S.nthreads > 0) omp_set_num_threads(S.nthreads);
#endif

  // the local grid of this (only) rank
  Domain::m_Ng_local_total = 1;
  for (int i = 0; i < 3; ++i) {
    Domain::m_ng_local_total[i] = S.ng[i];
    Domain::m_Ng_local_total *= S.ng[i];
  }
  std::vector<int> field(size_t(Domain::m_Ng_local_total) + 1, 0);

  alignas(Particles) static unsigned char storage[sizeof(Particles)];
  memset(storage, 0, sizeof(storage));
  Particles *P = reinterpret_cast<Particles *>(storage);
  P->m_xArr = a[0];
  P->m_yArr = a[1];
  P->m_zArr = a[2];
  P->m_vxArr = a[3];
  P->m_vyArr = a[4];
  P->m_vzArr = a[5];
  P->m_massArr = a[6];
  P->m_phiArr = a[7];
  P->m_idArr = id.data();
  P->m_maskArr = mask.data();
  P->m_field = reinterpret_cast<GRID_T *>(field.data());
  P->m_Np_local_total = int(n);
  P->m_Np_last = int(n);
  P->m_alpha = float(S.alpha);
  P->m_gpscal = S.gpscal;
  P->m_coords_localQ = 1;
  P->m_nsub = S.nsub;
  P->m_edge = S.edge;
  P->m_rsm = S.rsm;
  P->m_openAngle = S.open_angle;
  P->m_skipStreamQ = S.skip_stream;
  P->m_skipKickSRQ = S.skip_kick;
  P->m_useRCBTree = S.use_rcb_tree;
  P->m_rcbTreePPN = int(S.ppn);
  P->m_rcbTreeExtraLevels = int(S.extra_levels);
  P->m_rcbTreeTaskPartMin = int(S.task_part_min);
  // the polynomial short-range law, as Particles' constructor sets it with -P
  // (Particles.cxx:160-183)
  P->m_fg = new FGrid();
  P->m_fsrrmax = P->m_fg->rmax();
  P->m_fgore = new FGridEvalPoly(P->m_fg);
  P->m_fl = new ForceLawSR(P->m_fgore, P->m_rsm);

  TimeStepper ts(S.alpha, S.ain, S.afin, S.nsteps, S.omegatot);
  for (int h = 0; h < S.half_steps; ++h) ts.advanceHalfStep();
  const double pp = ts.pp(), aa = ts.aa(), zz = ts.zz(), adot = ts.adot(), tau = ts.tau(),
               tau2 = ts.tau2(), fscal = ts.fscal(), phiscal = ts.phiscal();
  if (S.nsub > 0) P->subCycle(&ts);

  FILE *o = fopen(argv[2], "wb");
  if (!o) { perror("open out"); return 2; }
  wr(o, "HSRSUBC1", 8);
  wr(o, &n, 1);
  wr(o, &S, 1);
  for (auto &v : a) if (n) wr(o, v, n);
  if (n) { wr(o, id.data(), n); wr(o, mask.data(), n); }
  fclose(o);
  printf("{\"pp\": %.17g, \"aa\": %.17g, \"zz\": %.17g, \"adot\": %.17g, \"tau\": %.17g, "
         "\"tau2\": %.17g, \"fscal\": %.17g, \"phiscal\": %.17g, \"np_last\": %d}\n",
         pp, aa, zz, adot, tau, tau2, fscal, phiscal, P->m_Np_last);
  return 0;
}
