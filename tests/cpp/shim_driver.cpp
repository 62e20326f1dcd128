// Calls the drop-in RCBForceTree / RCOForceTree (include/RCBForceTree_gb300.h,
// include/RCOForceTree_gb300.h) the way Particles::map2 constructs the
// reference trees, on one case file written by
// oracle/oracle.py (write_case), and writes the arrays back in the same format.
// Exit status 3 with a message when the library cannot run (no device).
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "RCBForceTree_gb300.h"
#include "RCOForceTree_gb300.h"

struct CaseParams {
  float min[3], max[3], min_force[3], max_force[3];
  float avg_mass, fsrrmax, rsm, open_angle;
  int64_t nd, ds, tmin;
  float fcoeff, ppc;
  int32_t tdpts, law, vmax, nthreads, reps, tree;
};

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  char magic[8];
  int64_t n = 0;
  CaseParams P;
  if (fread(magic, 1, 8, f) != 8 || fread(&n, 8, 1, f) != 1 || fread(&P, sizeof(P), 1, f) != 1) return 2;
  std::vector<float> a[8];
  for (auto &v : a) {
    v.resize(n);
    if (n && fread(v.data(), 4, n, f) != size_t(n)) return 2;
  }
  std::vector<int64_t> id(n);
  std::vector<uint16_t> mask(n);
  if (n && (fread(id.data(), 8, n, f) != size_t(n) || fread(mask.data(), 2, n, f) != size_t(n))) return 2;
  fclose(f);
  int token = 0;
  ForceLaw *fl = reinterpret_cast<ForceLaw *>(&token);  // stands for HACC's m_fl
  try {
    if (P.tree == 1) {
      hacc_sr_gb300::set_rco_softening(P.rsm);
      if (P.tdpts == 1) {
        RCOMonopoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, a[0].data(),
                               a[1].data(), a[2].data(), a[3].data(), a[4].data(), a[5].data(),
                               a[6].data(), a[7].data(), id.data(), mask.data(), P.avg_mass,
                               P.fsrrmax, P.open_angle, P.nd, P.ds, fl, P.fcoeff, P.ppc);
        printf("pairs %lld\n", (long long)t.stats().pairs);
      } else {
        RCOQuadrupoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, a[0].data(),
                                 a[1].data(), a[2].data(), a[3].data(), a[4].data(), a[5].data(),
                                 a[6].data(), a[7].data(), id.data(), mask.data(), P.avg_mass,
                                 P.fsrrmax, P.open_angle, P.nd, P.ds, fl, P.fcoeff, P.ppc);
        printf("pairs %lld\n", (long long)t.stats().pairs);
      }
    } else if (P.tdpts == 1) {
      RCBMonopoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, a[0].data(), a[1].data(),
                             a[2].data(), a[3].data(), a[4].data(), a[5].data(), a[6].data(),
                             a[7].data(), id.data(), mask.data(), P.avg_mass, P.fsrrmax, P.rsm,
                             P.open_angle, P.nd, P.ds, P.tmin, fl, P.fcoeff, P.ppc);
      printf("pairs %lld\n", (long long)t.stats().pairs);
    } else {
      RCBQuadrupoleForceTree t(P.min, P.max, P.min_force, P.max_force, n, a[0].data(),
                               a[1].data(), a[2].data(), a[3].data(), a[4].data(), a[5].data(),
                               a[6].data(), a[7].data(), id.data(), mask.data(), P.avg_mass,
                               P.fsrrmax, P.rsm, P.open_angle, P.nd, P.ds, P.tmin, fl, P.fcoeff,
                               P.ppc);
      printf("pairs %lld\n", (long long)t.stats().pairs);
    }
  } catch (const std::exception &e) {
    fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  fwrite("HSRCASE1", 1, 8, o);
  fwrite(&n, 8, 1, o);
  fwrite(&P, sizeof(P), 1, o);
  for (auto &v : a) if (n) fwrite(v.data(), 4, n, o);
  if (n) {
    fwrite(id.data(), 8, n, o);
    fwrite(mask.data(), 2, n, o);
  }
  fclose(o);
  return 0;
}
