// Calls the drop-in RCBForceTree / RCOForceTree (include/RCBForceTree_gb300.h,
// include/RCOForceTree_gb300.h) the way Particles::map2 constructs the
// reference trees, on one case file written by
// oracle/oracle.py (write_case), and writes the arrays back in the same format.
// Exit status 3 with a message when the library cannot run (no device) or
// refuses the force law.  An optional third argument picks the law passed as
// fl: "poly" (default; the polynomial short-range law at the case's
// softening), "fit" (the reference's FGridEvalFit law), "rsm" (the polynomial
// law at twice the softening) or "newton".
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "RCBForceTree_gb300.h"
#include "RCOForceTree_gb300.h"

// ForceLawSR::f_over_r over FGridEvalPoly (src/halo_finder/ForceLaw.cxx:
// 98-104, 187-192), in float.
struct PolyLaw : ForceLaw {
  float rsm2;
  explicit PolyLaw(float rsm) : rsm2(rsm * rsm) {}
  float f_over_r(float r2) override {
    const float a[7] = {0.271431f,    -0.0783394f,      0.0133122f,     -0.00159485f,
                        0.000132336f, -0.00000663394f, 0.000000147305f};
    const float p = a[0] + r2 * (a[1] + r2 * (a[2] + r2 * (a[3] + r2 * (a[4] + r2 * (a[5] + r2 * a[6])))));
    const float rmax = 3.116326355f;
    return (std::pow(r2 + rsm2, -1.5f) - p) * (r2 >= 0.f) * (r2 <= rmax * rmax);
  }
};

// ForceLawSR over FGridEvalFit: FGrid::fgor (src/halo_finder/ForceLaw.cxx:
// 23-52) evaluated at sqrt(r2), HACC's default law.
struct FitLaw : ForceLaw {
  float rsm2;
  explicit FitLaw(float rsm) : rsm2(rsm * rsm) {}
  static float fgor(float r) {
    const float b = 0.72f, c = 0.01f, d = 0.27f, e = 0.0001f, f = 360.0f, g = 100.0f, h = 0.67f,
                l = 17.0f, rmax = 3.116326355f;
    const float f0 = c + 2.0f / 3.0f * b * b * b;
    const float r2 = r * r, r4 = r2 * r2, r6 = r4 * r2;
    const float ch = std::cosh(b * r);
    const float r3 = std::tanh(b * r) - b * r / ch / ch + c * r * r2 * (1.0f + d * r2) * std::exp(-d * r2) +
                     e * r2 * (f * r2 + g * r4 + l * r6) * std::exp(-h * r2);
    const float rd = r + 1.0f * (r <= 0.f);
    return (r3 / (rd * rd * rd) + (r <= 0.f) * f0) * (r <= rmax) * (r >= 0.f);
  }
  float f_over_r(float r2) override {
    const float rmax = 3.116326355f;
    return (std::pow(r2 + rsm2, -1.5f) - fgor(std::sqrt(r2))) * (r2 >= 0.f) * (r2 <= rmax * rmax);
  }
};

struct NewtonLaw : ForceLaw {
  float f_over_r(float r2) override { return 1.0f / r2 / std::sqrt(r2); }
};

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
  const char *kind = argc > 3 ? argv[3] : "poly";
  PolyLaw poly(P.rsm), poly2(2.0f * P.rsm);
  FitLaw fit(P.rsm);
  NewtonLaw newton;
  ForceLaw *fl = &poly;  // stands for HACC's m_fl
  if (!strcmp(kind, "fit")) fl = &fit;
  if (!strcmp(kind, "rsm")) fl = &poly2;
  if (!strcmp(kind, "newton")) fl = &newton;
  try {
    if (P.tree == 1) {
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
