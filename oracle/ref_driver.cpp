// ref_driver.cpp -- runs the reference's own RCBForceTree (compiled unmodified
// from the reference sources by oracle/Makefile) on one case file.
//
// TEST INFRASTRUCTURE ONLY: used to pin the CPU restatement (hsr_oracle.c) and
// to write the golden fixtures.  Never part of the product.
//
// Usage: rcb_ref <case.bin> <out.bin>
// The case format is written by tests/hsr_case.py (write_case): an 8-byte
// magic "HSRCASE1", int64 n, the parameter block, then the ten particle arrays.
// The driver runs the constructor `reps` times on fresh copies of the input,
// writes the arrays after the last run, and prints one JSON line with the wall
// time of every run.  Needs a large stack (the reference keeps a VLA of n ints
// and four 16384-float lists on the stack): run it with an unlimited stack
// limit and OMP_STACKSIZE of a few hundred MB.
#include "ForceLaw.h"
#include "Partition.h"
#include "RCBForceTree.h"
#ifdef HSR_REF_RCO
#include "RCOForceTree.h"
#endif

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

// Storage for the Partition statics the force tree reads (rank number only).
int Partition::myProc = 0;
int Partition::numProc = 1;

namespace {

struct CaseParams {
  float min[3], max[3], min_force[3], max_force[3];
  float avg_mass, fsrrmax, rsm, open_angle;
  int64_t nd, ds, tmin;
  float fcoeff, ppc;
  int32_t tdpts, law, vmax, nthreads, reps;
  int32_t tree;  // 0: RCBForceTree; 1: RCOForceTree (builds with HSR_REF_RCO only)
};

template <typename T>
bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <typename T>
bool wr(FILE *f, const T *p, size_t n) { return fwrite(p, sizeof(T), n, f) == n; }

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s case.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror("open case"); return 2; }
  char magic[8];
  int64_t n = 0;
  CaseParams P;
  if (!rd(f, magic, 8) || memcmp(magic, "HSRCASE1", 8) != 0 || !rd(f, &n, 1) || !rd(f, &P, 1)) {
    fprintf(stderr, "bad case file\n");
    return 2;
  }
  std::vector<float> a[8];
  for (auto &v : a) { v.resize(n); if (n && !rd(f, v.data(), n)) return 2; }
  std::vector<int64_t> id(n);
  std::vector<uint16_t> mask(n);
  if (n && (!rd(f, id.data(), n) || !rd(f, mask.data(), n))) return 2;
  fclose(f);

  if (P.law != 0 || (P.tdpts != 1 && P.tdpts != 12)) {
    fprintf(stderr, "the reference generic path runs the 6th-order polynomial law with 1 or 12 pseudo-particles\n");
    return 3;
  }
#ifdef _OPENMP
  if (P.nthreads > 0) omp_set_num_threads(P.nthreads);
#endif

  FGrid fg;
  FGridEvalPoly fgore(&fg);
  ForceLawSR fl(&fgore, P.rsm);

  int reps = P.reps > 0 ? P.reps : 1;
  std::vector<float> w[8];
  std::vector<int64_t> wid;
  std::vector<uint16_t> wmask;
  std::vector<double> times;
  for (int r = 0; r < reps; ++r) {
    for (int k = 0; k < 8; ++k) w[k] = a[k];
    wid = id;
    wmask = mask;
    auto t0 = std::chrono::steady_clock::now();
#ifdef HSR_REF_RCO
    if (P.tree == 1 && P.tdpts == 1) {
      RCOMonopoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, w[0].data(), w[1].data(),
                             w[2].data(), w[3].data(), w[4].data(), w[5].data(), w[6].data(),
                             w[7].data(), wid.data(), wmask.data(), P.avg_mass, P.fsrrmax,
                             P.open_angle, P.nd, P.ds, &fl, P.fcoeff, P.ppc);
    } else if (P.tree == 1) {
      RCOQuadrupoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, w[0].data(),
                               w[1].data(), w[2].data(), w[3].data(), w[4].data(), w[5].data(),
                               w[6].data(), w[7].data(), wid.data(), wmask.data(), P.avg_mass,
                               P.fsrrmax, P.open_angle, P.nd, P.ds, &fl, P.fcoeff, P.ppc);
    } else
#else
    if (P.tree != 0) {
      fprintf(stderr, "this driver runs RCBForceTree only (build rco_ref for RCOForceTree)\n");
      return 3;
    }
#endif
    if (P.tdpts == 1) {
      RCBMonopoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, w[0].data(), w[1].data(),
                             w[2].data(), w[3].data(), w[4].data(), w[5].data(), w[6].data(),
                             w[7].data(), wid.data(), wmask.data(), P.avg_mass, P.fsrrmax, P.rsm,
                             P.open_angle, P.nd, P.ds, P.tmin, &fl, P.fcoeff, P.ppc);
    } else {
      RCBQuadrupoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, w[0].data(),
                               w[1].data(), w[2].data(), w[3].data(), w[4].data(), w[5].data(),
                               w[6].data(), w[7].data(), wid.data(), wmask.data(), P.avg_mass,
                               P.fsrrmax, P.rsm, P.open_angle, P.nd, P.ds, P.tmin, &fl, P.fcoeff,
                               P.ppc);
    }
    auto t1 = std::chrono::steady_clock::now();
    times.push_back(std::chrono::duration<double>(t1 - t0).count());
  }

  FILE *o = fopen(argv[2], "wb");
  if (!o) { perror("open out"); return 2; }
  wr(o, "HSRCASE1", 8);
  wr(o, &n, 1);
  wr(o, &P, 1);
  for (auto &v : w) if (n) wr(o, v.data(), n);
  if (n) { wr(o, wid.data(), n); wr(o, wmask.data(), n); }
  fclose(o);

  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  printf("{\"threads\": %d, \"times\": [", nth);
  for (size_t i = 0; i < times.size(); ++i) printf("%s%.6f", i ? ", " : "", times[i]);
  printf("]}\n");
  return 0;
}
