// pm.cu -- CIC deposit, quiet-solver spectra and inverse CIC kick for the
// long-range PM kick (reference pieces and the one-GPU layout in pm.cuh).
#include "pm.cuh"

#include <cmath>
#include <vector>

#include "device_info.cuh"

namespace hsr_pm {

namespace {

constexpr int kThreads = 256;

const char *cufft_name(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    default: return "cuFFT error";
  }
}

bool cu_ok(cudaError_t e, const char *what, std::string *err) {
  if (e == cudaSuccess) return true;
  *err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

bool fft_ok(cufftResult r, const char *what, std::string *err) {
  if (r == CUFFT_SUCCESS) return true;
  *err = std::string(what) + ": " + cufft_name(r);
  return false;
}

int blocks_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  const int64_t cap = int64_t(hsr::sm_count()) * 64;
  return int(b < cap ? (b > 0 ? b : 1) : cap);
}

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

// Alive-block index of local cell c (one axis), or -1 when the reference's
// deposit would land outside the alive block (dropped by
// fft_copy_arr_forward).
__device__ __forceinline__ int alive_cell(int c, int ngo, int ng) {
  const int u = c - ngo;
  return (u >= 0 && u < ng) ? u : -1;
}

// Periodic image in the alive block of local cell c, or -1 outside the local
// grid [0, nglt) (array_index's safe slot, value 0).  ngo + 1 <= ng, so one
// wrap suffices.
__device__ __forceinline__ int image_cell(int c, int ngo, int ng, int nglt) {
  if (c < 0 || c >= nglt) return -1;
  int u = c - ngo;
  if (u < 0) u += ng;
  else if (u >= ng) u -= ng;
  return u;
}

// Particles::cic (src/cpu/Particles.cxx:589-643) restricted to the alive
// block: ix = floor(x), weights ab = 1 + (ix - x), 1 - ab per axis, eight
// deposits of c * weight.
__global__ void __launch_bounds__(kThreads) k_cic(int64_t n, const float *__restrict__ x,
                                                  const float *__restrict__ y,
                                                  const float *__restrict__ z, int ng, int ngo,
                                                  int nglt, float c, float *__restrict__ rho) {
  const float lo = -2.0f, hi = float(nglt) + 1.0f;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float xx = x[i], yy = y[i], zz = z[i];
    // both cells of an axis lie outside [0, nglt) beyond these bounds (and
    // for NaN): nothing to deposit
    if (!(xx > lo && xx < hi && yy > lo && yy < hi && zz > lo && zz < hi)) continue;
    const int ix = int(floorf(xx)), iy = int(floorf(yy)), iz = int(floorf(zz));
    const float ab = 1.0f + (float(ix) - xx);
    const float de = 1.0f + (float(iy) - yy);
    const float gh = 1.0f + (float(iz) - zz);
    const int cx[2] = {alive_cell(ix, ngo, ng), alive_cell(ix + 1, ngo, ng)};
    const int cy[2] = {alive_cell(iy, ngo, ng), alive_cell(iy + 1, ngo, ng)};
    const int cz[2] = {alive_cell(iz, ngo, ng), alive_cell(iz + 1, ngo, ng)};
    const float wx[2] = {c * ab, c * (1.0f - ab)};
    const float wy[2] = {de, 1.0f - de};
    const float wz[2] = {gh, 1.0f - gh};
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      if (cx[a] < 0) continue;
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        if (cy[b] < 0) continue;
        const int64_t row = (int64_t(cx[a]) * ng + cy[b]) * ng;
        const float wxy = wx[a] * wy[b];
#pragma unroll
        for (int d = 0; d < 2; ++d)
          if (cz[d] >= 0) atomicAdd(rho + row + cz[d], wxy * wz[d]);
      }
    }
  }
}

// fft_copy_arr_forward (src/simulation/mc3.cxx:206-225): the alive block as
// the transform's real input.
__global__ void k_to_double(int64_t m, const float *__restrict__ a, double *__restrict__ b) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m;
       i += int64_t(gridDim.x) * blockDim.x)
    b[i] = double(a[i]);
}

// SolverQuiet's Green's function (src/dfft/solver.hpp:800-819) on the half
// spectrum, from the host's 1-D tables:
//   green = coeff * W(kx) * W(ky) * W(kz) / (d(kx) + d(ky) + d(kz)),
// coeff = 1 / ng^3, green(0) = 0.  Double products, sums and the division
// are correctly rounded on the device as on the host, so the values are the
// host loop's bit for bit.
template <typename T>
__global__ void k_green(int ng, int nh, const double *__restrict__ filter,
                        const double *__restrict__ denom, double coeff, T *__restrict__ green) {
  const int64_t m = int64_t(ng) * ng * nh;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int kz = int(i % nh);
    const int64_t t = i / nh;
    const int ky = int(t % ng), kx = int(t / ng);
    const double filt = __dmul_rn(__dmul_rn(__dmul_rn(coeff, filter[kx]), filter[ky]), filter[kz]);
    const double d = __dadd_rn(__dadd_rn(denom[kx], denom[ky]), denom[kz]);
    green[i] = (i == 0) ? T(0) : T(filt / d);
  }
}

// SolverBase::kspace_solve_gradient (src/dfft/solver.hpp:506-547) for the
// three axes at once: grad_a = I * (-g(k_a)) * green * rho_k, i.e.
// (t * Im rho, -t * Re rho) with t = g(k_a) * green.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_spectra(int ng, int nh, const typename Cplx<T>::type *__restrict__ rho,
              const T *__restrict__ green, const T *__restrict__ g,
              typename Cplx<T>::type *__restrict__ out) {
  using C = typename Cplx<T>::type;
  const int64_t m = int64_t(ng) * ng * nh;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int kz = int(i % nh);
    const int64_t t = i / nh;
    const int ky = int(t % ng), kx = int(t / ng);
    const T G = green[i];
    const C r = rho[i];
    const int k[3] = {kx, ky, kz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const T s = g[k[a]] * G;
      C o;
      o.x = s * r.y;
      o.y = -(s * r.x);
      out[a * m + i] = o;
    }
  }
}

// fft_copy_arr_backward (src/simulation/mc3.cxx:228-245) of the three
// components: float(real part) into one float4 per cell.
template <typename T>
__global__ void k_pack(int64_t m, const T *__restrict__ g, float4 *__restrict__ out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m;
       i += int64_t(gridDim.x) * blockDim.x)
    out[i] = make_float4(float(g[i]), float(g[m + i]), float(g[2 * m + i]), 0.0f);
}

// Particles::inverse_cic (src/cpu/Particles.cxx:647-714) for the three
// components in one pass, the corners in the reference's order; each local
// cell reads its periodic image (GridExchange on one rank), cells outside
// the local grid read 0.
__global__ void __launch_bounds__(kThreads)
    k_cic_inv(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
              const float *__restrict__ z, int ng, int ngo, int nglt,
              const float4 *__restrict__ grad, float fscal, float tau, float *__restrict__ vx,
              float *__restrict__ vy, float *__restrict__ vz) {
  const float lo = -2.0f, hi = float(nglt) + 1.0f;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float xx = x[i], yy = y[i], zz = z[i];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if (xx > lo && xx < hi && yy > lo && yy < hi && zz > lo && zz < hi) {
      const int ix = int(floorf(xx)), iy = int(floorf(yy)), iz = int(floorf(zz));
      const float ab = 1.0f + (float(ix) - xx);
      const float de = 1.0f + (float(iy) - yy);
      const float gh = 1.0f + (float(iz) - zz);
      const int cx[2] = {image_cell(ix, ngo, ng, nglt), image_cell(ix + 1, ngo, ng, nglt)};
      const int cy[2] = {image_cell(iy, ngo, ng, nglt), image_cell(iy + 1, ngo, ng, nglt)};
      const int cz[2] = {image_cell(iz, ngo, ng, nglt), image_cell(iz + 1, ngo, ng, nglt)};
      const float wx[2] = {ab, 1.0f - ab};
      const float wy[2] = {de, 1.0f - de};
      const float wz[2] = {gh, 1.0f - gh};
      // (ix,iy,iz) (ix,jp,iz) (ix,jp,kp) (ix,iy,kp) (ip,iy,kp) (ip,jp,kp) (ip,jp,iz) (ip,iy,iz)
      const int order[8][3] = {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1},
                               {1, 0, 1}, {1, 1, 1}, {1, 1, 0}, {1, 0, 0}};
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int a = order[q][0], b = order[q][1], d = order[q][2];
        if (cx[a] < 0 || cy[b] < 0 || cz[d] < 0) continue;
        const float4 v = __ldg(grad + (int64_t(cx[a]) * ng + cy[b]) * ng + cz[d]);
        const float w = wx[a] * wy[b] * wz[d];
        fx += v.x * w;
        fy += v.y * w;
        fz += v.z * w;
      }
    }
    vx[i] += fx * fscal * tau;
    vy[i] += fy * fscal * tau;
    vz[i] += fz * fscal * tau;
  }
}

// The CIC weights of a particle and their derivatives, the corner cells
// mapped as `map` says (-1: no cell).  Returns false when every corner lies
// outside the local grid (and for NaN).
struct Cic {
  int cx[2], cy[2], cz[2];
  float wx[2], wy[2], wz[2];
};

__device__ __forceinline__ bool cic_of(float xx, float yy, float zz, int nglt, Cic &c, int *ix3) {
  const float lo = -2.0f, hi = float(nglt) + 1.0f;
  if (!(xx > lo && xx < hi && yy > lo && yy < hi && zz > lo && zz < hi)) return false;
  const int ix = int(floorf(xx)), iy = int(floorf(yy)), iz = int(floorf(zz));
  const float ab = 1.0f + (float(ix) - xx);
  const float de = 1.0f + (float(iy) - yy);
  const float gh = 1.0f + (float(iz) - zz);
  c.wx[0] = ab;
  c.wx[1] = 1.0f - ab;
  c.wy[0] = de;
  c.wy[1] = 1.0f - de;
  c.wz[0] = gh;
  c.wz[1] = 1.0f - gh;
  ix3[0] = ix;
  ix3[1] = iy;
  ix3[2] = iz;
  return true;
}

// Transpose of the interpolation for the three cotangent components:
// adj_a[image(c)] += W(x - c) vbar_a.
__global__ void __launch_bounds__(kThreads)
    k_adj_deposit(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
                  const float *__restrict__ z, const float *__restrict__ vbx,
                  const float *__restrict__ vby, const float *__restrict__ vbz, int ng, int ngo,
                  int nglt, float *__restrict__ adj) {
  const int64_t m = int64_t(ng) * ng * ng;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    Cic c;
    int i3[3];
    if (!cic_of(x[i], y[i], z[i], nglt, c, i3)) continue;
    const float u[3] = {vbx[i], vby[i], vbz[i]};
    int cx[2], cy[2], cz[2];
    for (int a = 0; a < 2; ++a) {
      cx[a] = image_cell(i3[0] + a, ngo, ng, nglt);
      cy[a] = image_cell(i3[1] + a, ngo, ng, nglt);
      cz[a] = image_cell(i3[2] + a, ngo, ng, nglt);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      if (cx[a] < 0) continue;
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        if (cy[b] < 0) continue;
        const int64_t row = (int64_t(cx[a]) * ng + cy[b]) * ng;
        const float wab = c.wx[a] * c.wy[b];
#pragma unroll
        for (int d = 0; d < 2; ++d) {
          if (cz[d] < 0) continue;
          const float w = wab * c.wz[d];
          const int64_t k = row + cz[d];
          atomicAdd(adj + k, w * u[0]);
          atomicAdd(adj + m + k, w * u[1]);
          atomicAdd(adj + 2 * m + k, w * u[2]);
        }
      }
    }
  }
}

template <typename T>
__global__ void k_to_real3(int64_t m3, const float *__restrict__ a, T *__restrict__ b) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m3;
       i += int64_t(gridDim.x) * blockDim.x)
    b[i] = T(a[i]);
}

// The transposed solve, summed over the three components:
// phibar_k = sum_a conj(S_a) adj_a,k with S_a = -I g(k_a) green, i.e.
// green * sum_a I g(k_a) adj_a,k.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_adj_spectra(int ng, int nh, const typename Cplx<T>::type *__restrict__ a3,
                  const T *__restrict__ green, const T *__restrict__ g,
                  typename Cplx<T>::type *__restrict__ out) {
  using C = typename Cplx<T>::type;
  const int64_t m = int64_t(ng) * ng * nh;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int kz = int(i % nh);
    const int64_t t = i / nh;
    const int ky = int(t % ng), kx = int(t / ng);
    const int k[3] = {kx, ky, kz};
    T re = T(0), im = T(0);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const C v = a3[a * m + i];
      const T ga = g[k[a]];
      re -= ga * v.y;
      im += ga * v.x;
    }
    const T G = green[i];
    C o;
    o.x = G * re;
    o.y = G * im;
    out[i] = o;
  }
}

// xbar = fscal tau [sum_c grad W (vbar . G[image(c)])
//                   + gpscal^3 sum_{c alive} grad W phibar[c]].
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_vjp_interp(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
                 const float *__restrict__ z, const float *__restrict__ vbx,
                 const float *__restrict__ vby, const float *__restrict__ vbz, int ng, int ngo,
                 int nglt, const float4 *__restrict__ grad, const T *__restrict__ phibar,
                 float cm, float coef, float *__restrict__ xbx, float *__restrict__ xby,
                 float *__restrict__ xbz) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    float gx = 0.f, gy = 0.f, gz = 0.f;
    Cic c;
    int i3[3];
    if (cic_of(x[i], y[i], z[i], nglt, c, i3)) {
      const float u0 = vbx[i], u1 = vby[i], u2 = vbz[i];
      const float sg[2] = {-1.0f, 1.0f};
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            const float dwx = sg[a] * c.wy[b] * c.wz[d];
            const float dwy = c.wx[a] * sg[b] * c.wz[d];
            const float dwz = c.wx[a] * c.wy[b] * sg[d];
            float f = 0.f;
            const int ix = image_cell(i3[0] + a, ngo, ng, nglt);
            const int iy = image_cell(i3[1] + b, ngo, ng, nglt);
            const int iz = image_cell(i3[2] + d, ngo, ng, nglt);
            if (ix >= 0 && iy >= 0 && iz >= 0) {
              const float4 G = __ldg(grad + (int64_t(ix) * ng + iy) * ng + iz);
              f = fmaf(u0, G.x, fmaf(u1, G.y, u2 * G.z));
            }
            const int ax = alive_cell(i3[0] + a, ngo, ng);
            const int ay = alive_cell(i3[1] + b, ngo, ng);
            const int az = alive_cell(i3[2] + d, ngo, ng);
            if (ax >= 0 && ay >= 0 && az >= 0)
              f = fmaf(cm, float(phibar[(int64_t(ax) * ng + ay) * ng + az]), f);
            gx = fmaf(dwx, f, gx);
            gy = fmaf(dwy, f, gy);
            gz = fmaf(dwz, f, gz);
          }
    }
    xbx[i] = coef * gx;
    xby[i] = coef * gy;
    xbz[i] = coef * gz;
  }
}

}  // namespace

void quiet_tables(int ng, double *filter, double *denom, double *gradient) {
  // src/dfft/solver.hpp:33, 726-790
  const double pi = 3.14159265358979323846;
  const double a0 = -21.0 / 8.0, a1 = 128.0 / 45.0, a2 = -2.0 / 9.0, a3 = 1.0 / 360.0;
  const double b1 = 4.0 / 3.0, b2 = -1.0 / 6.0;
  const double sigma = 0.8, ns = 3.0;
  std::vector<double> c1(ng), c2(ng), c3(ng), kp(ng, 0.0);
  const double kstep = 2.0 * pi / static_cast<double>(ng);
  for (int kk = 0; kk < ng; ++kk) {
    c1[kk] = std::cos(kk * kstep);
    c2[kk] = std::cos(2 * kk * kstep);
    c3[kk] = std::cos(4 * kk * kstep);
    if (kk < ng / 2) {
      kp[kk] = kk * kstep;
      kp[kk + ng / 2] = (kk - ng / 2) * kstep;
    }
  }
  filter[0] = 1.0;
  gradient[0] = 1.0;
  for (int kk = 1; kk < ng; ++kk) {
    filter[kk] = std::exp(-0.25 * sigma * sigma * kp[kk] * kp[kk]) *
                 std::pow(std::sin(0.5 * kp[kk]) / (0.5 * kp[kk]), ns);
    gradient[kk] = (b1 * std::sin(kp[kk]) + b2 * std::sin(2 * kp[kk]));
  }
  for (int kk = 0; kk < ng; ++kk) denom[kk] = a0 + a1 * c1[kk] + a2 * c2[kk] + a3 * c3[kk];
}

Solver::~Solver() { release(); }

void Solver::release() {
  if (have_fwd_) cufftDestroy(fwd_);
  if (have_inv_) cufftDestroy(inv_);
  if (have_fwd3_) cufftDestroy(fwd3_);
  if (have_inv1_) cufftDestroy(inv1_);
  have_fwd_ = have_inv_ = have_fwd3_ = have_inv1_ = false;
  for (void *p : {(void *)rho_, real_, spec_, gspec_, greal_, green_, gtab_, (void *)grad_,
                  (void *)adj_})
    if (p) cudaFree(p);
  rho_ = adj_ = nullptr;
  real_ = spec_ = gspec_ = greal_ = green_ = gtab_ = nullptr;
  grad_ = nullptr;
  ng_ = 0;
  prec_ = -1;
}

bool Solver::prepare(int ng, int prec, cudaStream_t s, std::string *err) {
  if (ng == ng_ && prec == prec_) return true;
  release();
  const int nh = ng / 2 + 1;
  const int64_t m = int64_t(ng) * ng * ng, mh = int64_t(ng) * ng * nh;
  const size_t rs = prec == PREC_F64 ? sizeof(double) : sizeof(float);
  const size_t cs = 2 * rs;
  if (!cu_ok(cudaMalloc(&rho_, m * sizeof(float)), "pm rho", err)) return release(), false;
  if (prec == PREC_F64 && !cu_ok(cudaMalloc(&real_, m * rs), "pm real", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&spec_, mh * cs), "pm spectrum", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&gspec_, 3 * mh * cs), "pm gradient spectra", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&greal_, 3 * m * rs), "pm gradient fields", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&green_, mh * rs), "pm green", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&gtab_, ng * rs), "pm gradient table", err)) return release(), false;
  if (!cu_ok(cudaMalloc(&grad_, m * sizeof(float4)), "pm gradient grid", err)) return release(), false;

  // tables (host, double) -> Green's function (device)
  std::vector<double> filter(ng), denom(ng), gradient(ng);
  quiet_tables(ng, filter.data(), denom.data(), gradient.data());
  // the real part the reference keeps gets nothing from the planes k_a = 0
  // and k_a = ng / 2 of the gradient axis (pm.cuh)
  gradient[0] = 0.0;
  gradient[ng / 2] = 0.0;
  double *d_tab = nullptr;
  if (!cu_ok(cudaMalloc(&d_tab, 2 * ng * sizeof(double)), "pm tables", err)) return release(), false;
  std::vector<double> both(filter);
  both.insert(both.end(), denom.begin(), denom.end());
  bool ok = cu_ok(cudaMemcpyAsync(d_tab, both.data(), 2 * ng * sizeof(double), cudaMemcpyHostToDevice, s),
                  "pm tables copy", err);
  const double coeff = 1.0 / double(m);
  if (ok) {
    if (prec == PREC_F64)
      k_green<double><<<blocks_for(mh), kThreads, 0, s>>>(ng, nh, d_tab, d_tab + ng, coeff,
                                                          (double *)green_);
    else
      k_green<float><<<blocks_for(mh), kThreads, 0, s>>>(ng, nh, d_tab, d_tab + ng, coeff,
                                                         (float *)green_);
    ok = cu_ok(cudaGetLastError(), "pm green kernel", err);
  }
  if (ok) {
    if (prec == PREC_F64) {
      ok = cu_ok(cudaMemcpyAsync(gtab_, gradient.data(), ng * sizeof(double), cudaMemcpyHostToDevice, s),
                 "pm gradient table copy", err);
    } else {
      std::vector<float> gf(gradient.begin(), gradient.end());
      ok = cu_ok(cudaMemcpyAsync(gtab_, gf.data(), ng * sizeof(float), cudaMemcpyHostToDevice, s),
                 "pm gradient table copy", err);
      if (ok) ok = cu_ok(cudaStreamSynchronize(s), "pm tables", err);
    }
  }
  if (ok) ok = cu_ok(cudaStreamSynchronize(s), "pm tables", err);
  cudaFree(d_tab);
  if (!ok) return release(), false;

  // plans (64-bit sizes): one forward real-to-complex transform, one
  // batched inverse of the three gradient spectra
  long long dims[3] = {ng, ng, ng};
  const bool f64 = prec == PREC_F64;
  size_t ws = 0;
  if (!fft_ok(cufftCreate(&fwd_), "pm forward plan", err)) return release(), false;
  have_fwd_ = true;
  if (!fft_ok(cufftMakePlanMany64(fwd_, 3, dims, nullptr, 1, m, nullptr, 1, mh,
                                  f64 ? CUFFT_D2Z : CUFFT_R2C, 1, &ws),
              "pm forward plan", err))
    return release(), false;
  if (!fft_ok(cufftCreate(&inv_), "pm inverse plan", err)) return release(), false;
  have_inv_ = true;
  if (!fft_ok(cufftMakePlanMany64(inv_, 3, dims, nullptr, 1, mh, nullptr, 1, m,
                                  f64 ? CUFFT_Z2D : CUFFT_C2R, 3, &ws),
              "pm inverse plan", err))
    return release(), false;
  ng_ = ng;
  prec_ = prec;
  return true;
}

bool Solver::deposit(const Params &p, int64_t n, const float *x, const float *y, const float *z,
                     cudaStream_t s, std::string *err) {
  const int ng = p.ng;
  const int64_t m = int64_t(ng) * ng * ng;
  if (!cu_ok(cudaMemsetAsync(rho_, 0, m * sizeof(float), s), "pm rho clear", err)) return false;
  if (n > 0) {
    const float c = p.gpscal * p.gpscal * p.gpscal;  // Particles.cxx:605
    k_cic<<<blocks_for(n), kThreads, 0, s>>>(n, x, y, z, ng, p.ngo, ng + 2 * p.ngo + 1, c, rho_);
    ++launches;
    if (!cu_ok(cudaGetLastError(), "pm cic kernel", err)) return false;
  }
  return true;
}

bool Solver::solve(cudaStream_t s, std::string *err) {
  const int ng = ng_, nh = ng / 2 + 1;
  const int64_t m = int64_t(ng) * ng * ng, mh = int64_t(ng) * ng * nh;
  if (!fft_ok(cufftSetStream(fwd_, s), "pm forward stream", err)) return false;
  if (!fft_ok(cufftSetStream(inv_, s), "pm inverse stream", err)) return false;
  if (prec_ == PREC_F64) {
    k_to_double<<<blocks_for(m), kThreads, 0, s>>>(m, rho_, (double *)real_);
    ++launches;
    if (!cu_ok(cudaGetLastError(), "pm copy forward", err)) return false;
    if (!fft_ok(cufftExecD2Z(fwd_, (cufftDoubleReal *)real_, (cufftDoubleComplex *)spec_),
                "pm forward transform", err))
      return false;
    k_spectra<double><<<blocks_for(mh), kThreads, 0, s>>>(ng, nh, (const double2 *)spec_,
                                                          (const double *)green_,
                                                          (const double *)gtab_, (double2 *)gspec_);
    ++launches;
    if (!cu_ok(cudaGetLastError(), "pm spectra kernel", err)) return false;
    if (!fft_ok(cufftExecZ2D(inv_, (cufftDoubleComplex *)gspec_, (cufftDoubleReal *)greal_),
                "pm inverse transform", err))
      return false;
    k_pack<double><<<blocks_for(m), kThreads, 0, s>>>(m, (const double *)greal_, grad_);
  } else {
    if (!fft_ok(cufftExecR2C(fwd_, (cufftReal *)rho_, (cufftComplex *)spec_), "pm forward transform",
                err))
      return false;
    k_spectra<float><<<blocks_for(mh), kThreads, 0, s>>>(ng, nh, (const float2 *)spec_,
                                                         (const float *)green_,
                                                         (const float *)gtab_, (float2 *)gspec_);
    ++launches;
    if (!cu_ok(cudaGetLastError(), "pm spectra kernel", err)) return false;
    if (!fft_ok(cufftExecC2R(inv_, (cufftComplex *)gspec_, (cufftReal *)greal_),
                "pm inverse transform", err))
      return false;
    k_pack<float><<<blocks_for(m), kThreads, 0, s>>>(m, (const float *)greal_, grad_);
  }
  ++launches;
  fft_execs += 2;
  return cu_ok(cudaGetLastError(), "pm pack kernel", err);
}

bool Solver::interp(const Params &p, int64_t n, const float *x, const float *y, const float *z,
                    float *vx, float *vy, float *vz, cudaStream_t s, std::string *err) {
  if (n == 0) return true;
  k_cic_inv<<<blocks_for(n), kThreads, 0, s>>>(n, x, y, z, p.ng, p.ngo, p.ng + 2 * p.ngo + 1,
                                               grad_, p.fscal, p.tau, vx, vy, vz);
  ++launches;
  return cu_ok(cudaGetLastError(), "pm inverse cic kernel", err);
}

bool Solver::export_fields(float *rho, float *grad, bool to_host, cudaStream_t s, std::string *err) {
  const int64_t m = int64_t(ng_) * ng_ * ng_;
  const cudaMemcpyKind k = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (rho && !cu_ok(cudaMemcpyAsync(rho, rho_, m * sizeof(float), k, s), "pm rho export", err))
    return false;
  if (grad) {
    // float4 cells -> three planar components
    for (int a = 0; a < 3; ++a)
      if (!cu_ok(cudaMemcpy2DAsync(grad + a * m, sizeof(float), (const float *)grad_ + a,
                                   sizeof(float4), sizeof(float), m, k, s),
                 "pm gradient export", err))
        return false;
  }
  return cu_ok(cudaStreamSynchronize(s), "pm export", err);
}

bool Solver::prepare_vjp(std::string *err) {
  if (have_fwd3_ && have_inv1_ && adj_) return true;
  const int ng = ng_, nh = ng / 2 + 1;
  const int64_t m = int64_t(ng) * ng * ng, mh = int64_t(ng) * ng * nh;
  if (!adj_ && !cu_ok(cudaMalloc(&adj_, 3 * m * sizeof(float)), "pm adjoint fields", err))
    return false;
  long long dims[3] = {ng, ng, ng};
  const bool f64 = prec_ == PREC_F64;
  size_t ws = 0;
  if (!have_fwd3_) {
    if (!fft_ok(cufftCreate(&fwd3_), "pm adjoint forward plan", err)) return false;
    have_fwd3_ = true;
    if (!fft_ok(cufftMakePlanMany64(fwd3_, 3, dims, nullptr, 1, m, nullptr, 1, mh,
                                    f64 ? CUFFT_D2Z : CUFFT_R2C, 3, &ws),
                "pm adjoint forward plan", err))
      return false;
  }
  if (!have_inv1_) {
    if (!fft_ok(cufftCreate(&inv1_), "pm adjoint inverse plan", err)) return false;
    have_inv1_ = true;
    if (!fft_ok(cufftMakePlanMany64(inv1_, 3, dims, nullptr, 1, mh, nullptr, 1, m,
                                    f64 ? CUFFT_Z2D : CUFFT_C2R, 1, &ws),
                "pm adjoint inverse plan", err))
      return false;
  }
  return true;
}

bool Solver::vjp(const Params &p, int64_t n, const float *x, const float *y, const float *z,
                 const float *vbx, const float *vby, const float *vbz, float *xbx, float *xby,
                 float *xbz, cudaStream_t s, std::string *err) {
  if (!prepare_vjp(err)) return false;
  if (!deposit(p, n, x, y, z, s, err) || !solve(s, err)) return false;
  if (n == 0) return true;
  const int ng = ng_, nh = ng / 2 + 1, nglt = ng + 2 * p.ngo + 1;
  const int64_t m = int64_t(ng) * ng * ng, mh = int64_t(ng) * ng * nh;
  if (!cu_ok(cudaMemsetAsync(adj_, 0, 3 * m * sizeof(float), s), "pm adjoint clear", err))
    return false;
  k_adj_deposit<<<blocks_for(n), kThreads, 0, s>>>(n, x, y, z, vbx, vby, vbz, ng, p.ngo, nglt,
                                                   adj_);
  ++launches;
  if (!cu_ok(cudaGetLastError(), "pm adjoint deposit", err)) return false;
  if (!fft_ok(cufftSetStream(fwd3_, s), "pm adjoint stream", err)) return false;
  if (!fft_ok(cufftSetStream(inv1_, s), "pm adjoint stream", err)) return false;
  const float cm = p.gpscal * p.gpscal * p.gpscal;
  const float coef = p.fscal * p.tau;
  if (prec_ == PREC_F64) {
    k_to_real3<double><<<blocks_for(3 * m), kThreads, 0, s>>>(3 * m, adj_, (double *)greal_);
    if (!fft_ok(cufftExecD2Z(fwd3_, (cufftDoubleReal *)greal_, (cufftDoubleComplex *)gspec_),
                "pm adjoint forward transform", err))
      return false;
    k_adj_spectra<double><<<blocks_for(mh), kThreads, 0, s>>>(
        ng, nh, (const double2 *)gspec_, (const double *)green_, (const double *)gtab_,
        (double2 *)spec_);
    if (!fft_ok(cufftExecZ2D(inv1_, (cufftDoubleComplex *)spec_, (cufftDoubleReal *)real_),
                "pm adjoint inverse transform", err))
      return false;
    k_vjp_interp<double><<<blocks_for(n), kThreads, 0, s>>>(
        n, x, y, z, vbx, vby, vbz, ng, p.ngo, nglt, grad_, (const double *)real_, cm, coef, xbx,
        xby, xbz);
  } else {
    if (!fft_ok(cufftExecR2C(fwd3_, (cufftReal *)adj_, (cufftComplex *)gspec_),
                "pm adjoint forward transform", err))
      return false;
    k_adj_spectra<float><<<blocks_for(mh), kThreads, 0, s>>>(
        ng, nh, (const float2 *)gspec_, (const float *)green_, (const float *)gtab_,
        (float2 *)spec_);
    // the density grid is free once the solve ran: the inverse lands there
    if (!fft_ok(cufftExecC2R(inv1_, (cufftComplex *)spec_, (cufftReal *)rho_),
                "pm adjoint inverse transform", err))
      return false;
    k_vjp_interp<float><<<blocks_for(n), kThreads, 0, s>>>(n, x, y, z, vbx, vby, vbz, ng, p.ngo,
                                                          nglt, grad_, rho_, cm, coef, xbx, xby,
                                                          xbz);
  }
  launches += prec_ == PREC_F64 ? 3 : 2;
  fft_execs += 2;
  return cu_ok(cudaGetLastError(), "pm adjoint kernels", err);
}

bool Solver::kick(const Params &p, int64_t n, const float *x, const float *y, const float *z,
                  float *vx, float *vy, float *vz, cudaStream_t s, cudaEvent_t *ev, Timing *t,
                  std::string *err) {
  const int64_t l0 = launches, f0 = fft_execs;
  if (!cu_ok(cudaEventRecord(ev[0], s), "pm event", err)) return false;
  if (!deposit(p, n, x, y, z, s, err)) return false;
  if (!cu_ok(cudaEventRecord(ev[1], s), "pm event", err)) return false;
  if (!solve(s, err)) return false;
  if (!cu_ok(cudaEventRecord(ev[2], s), "pm event", err)) return false;
  if (!interp(p, n, x, y, z, vx, vy, vz, s, err)) return false;
  if (!cu_ok(cudaEventRecord(ev[3], s), "pm event", err)) return false;
  if (!cu_ok(cudaEventSynchronize(ev[3]), "pm kick", err)) return false;
  float a = 0, b = 0, c = 0;
  cudaEventElapsedTime(&a, ev[0], ev[1]);
  cudaEventElapsedTime(&b, ev[1], ev[2]);
  cudaEventElapsedTime(&c, ev[2], ev[3]);
  t->deposit_ms = a;
  t->solve_ms = b;
  t->interp_ms = c;
  t->launches = launches - l0;
  t->fft_execs = fft_execs - f0;
  return true;
}

}  // namespace hsr_pm
