// kernels_place.cu -- per-placement solute preparation and the plain FP64 PME path.
//
//   place_prep    solute sites of every placement in a batch: wrapped FP64 and
//                 fixed-point coordinates, calc_spline_molecule (recpcal.F90:408-442,
//                 FP64 weights on both paths),
//                 realcal_self (realcal.F90:284-328, FP64) and, for the mixed path,
//                 the 1-D structure-factor vectors
//                     b_{s,a}(k) = sum_c theta_{s,a,c} exp(-2 pi i k (g_{s,a} - c) / K_a);
//                 (the mixed path's spectrum and transforms are in kernels_fft.cu);
//   spread64 / influence64   the plain FP64 path, literally the reference's order:
//                 spread, D2Z (cuFFT), self energy + engfac multiply, Z2D (cuFFT).
#include "engine.cuh"

namespace ermod {

namespace {

__host__ __device__ __forceinline__ double ipow_d(double x, int e) {
  double r = 1.0;
  bool first = true;
  while (e > 0) {
    if (e & 1) {
      r = first ? x : r * x;
      first = false;
    }
    e >>= 1;
    if (e) x = x * x;
  }
  return r;
}

struct Coef {
  double c[kMaxSplineOrder + 1];
  int order;
  double screen;
};

__device__ __forceinline__ double spline_value(const Coef& s, double rst) {  // spline.F90:47-59
  double f = 0.0;
  if ((rst > 0.0) && (rst < (double)s.order)) {
    const int k = (int)rst;
    for (int i = 0; i <= k; ++i) f = f + s.c[i] * ipow_d(rst - (double)i, s.order - 1);
  }
  return f;
}

struct PrepArgs {
  BatchArgs a;
  const double* solxyz;   // [nb][S][3] raw solute coordinates of this batch, or null (use frame)
  const double* sitepos;  // frame raw coordinates
  const int* mbi0;        // [nummol+1] 0-based
  const double* charge;
  const int* ljtype;
  const double* mol_qmol_all;  // [nummol]
  const double2* twiddle64;    // [K1+K2+K3] exp(-2 pi i m / K)
  FrameGeom g;
  Coef sc;
  int mixed;
  int self_mode;  // 0: none, 1: all placements, 2: only placement 0 of the batch
  int nummol;
  int bare;  // cltype 0
  unsigned mK[3], mKmax, m3Kmax;  // ceil(2^32 / d): n / d = umulhi(n, m) for n d < 2^32
  DevStatus* status;
};

__device__ __forceinline__ void wrap_coord(const double* v, double x0raw, const FrameGeom& g, double out[3]) {
  for (int i = 0; i < 3; ++i) out[i] = v[i] - g.L[i] * floor(g.invL[i] * v[i]);
  out[1] = out[1] - g.L[1] * floor(g.invL[1] * out[1]);
  const double x0 = x0raw - g.L[0] * floor(g.invL[0] * x0raw);
  const double x0b = x0 - g.L[0] * floor(g.invL[0] * x0);
  out[0] = out[0] - g.L[0] * floor(g.invL[0] * x0b);
}

// one block per placement of the batch
__global__ void __launch_bounds__(256) place_prep_kernel(PrepArgs A) {
  const int b = blockIdx.x;
  const BatchArgs& a = A.a;
  const FrameGeom& g = A.g;
  const int mol = a.tagslt[b] - 1;
  if (mol < 0 || mol >= A.nummol) {  // device-side inputs are checked here, not trusted
    if (threadIdx.x == 0) {
      atomicOr(&A.status->range_fault, 1);
      a.u_nsite[b] = 0;
    }
    return;
  }
  const int atom0 = A.mbi0[mol];
  const int ns = A.mbi0[mol + 1] - atom0;
  const int P = A.sc.order;
  __shared__ double sx[kMaxSoluteSites][3];
  __shared__ double red[256];
  __shared__ int sgrd[kMaxSoluteSites][3];
  if (ns > kMaxSoluteSites) {
    if (threadIdx.x == 0) {
      atomicOr(&A.status->range_fault, 1);
      a.u_nsite[b] = 0;
    }
    return;
  }
  for (int s = threadIdx.x; s < ns; s += blockDim.x) {
    const double* raw = A.solxyz ? A.solxyz + ((size_t)b * ns + s) * 3 : A.sitepos + 3 * (size_t)(atom0 + s);
    double w[3];
    const bool is_atom1 = (A.solxyz == nullptr) && (atom0 + s == 0);
    if (!g.periodic) {  // non-periodic: coordinates as they are, within the fixed-point reach
      for (int i = 0; i < 3; ++i) {
        w[i] = raw[i];
        if (!(fabs(raw[i]) < g.reach)) atomicOr(&A.status->range_fault, 4);
      }
    } else if (is_atom1) {  // atom 1 itself takes the first-pass x shift of its own x
      for (int i = 0; i < 3; ++i) w[i] = raw[i] - g.L[i] * floor(g.invL[i] * raw[i]);
      w[1] = w[1] - g.L[1] * floor(g.invL[1] * w[1]);
      w[0] = w[0] - g.L[0] * floor(g.invL[0] * w[0]);
    } else {
      wrap_coord(raw, A.sitepos[0], g, w);
    }
    const size_t us = (size_t)b * kMaxSoluteSites + s;
    for (int i = 0; i < 3; ++i) {
      a.u_x[us * 3 + i] = w[i];
      sx[s][i] = w[i];
    }
    unsigned int X[3];
    for (int i = 0; i < 3; ++i) X[i] = (unsigned int)(unsigned long long)llrint(w[i] * g.invL[i] * 4294967296.0);
    a.u_pos[us] = make_int4((int)X[0], (int)X[1], (int)X[2], A.ljtype[atom0 + s]);
    a.u_q[us] = A.charge[atom0 + s];
    a.u_qf[us] = (float)A.charge[atom0 + s];
    int rci[3];
    for (int kk = 0; kk < 3; ++kk) {  // calc_spline_molecule on the raw coordinates
      double factor = g.invcl[kk + 0] * raw[0] + g.invcl[kk + 3] * raw[1] + g.invcl[kk + 6] * raw[2];
      factor = factor - floor(factor);
      const double f2 = factor * (double)g.K[kk];
      rci[kk] = (int)f2;
      double* uw = a.u_w + (us * 3 + kk) * kMaxSplineOrder;
      // FP64 weights on both paths: on the mixed path they set the 1-D structure factors,
      // whose accuracy bounds that of the solute self energy (the weights of placements)
      for (int spi = 0; spi < P; ++spi) uw[spi] = spline_value(A.sc, f2 - (double)(rci[kk] - spi));
      sgrd[s][kk] = rci[kk];
    }
    a.u_grid[us] = rci[0] | (rci[1] << kGridBits) | (rci[2] << (2 * kGridBits));
  }
  if (threadIdx.x == 0) {
    a.u_nsite[b] = ns;
    a.u_qmol[b] = A.mol_qmol_all[mol];
  }
  __syncthreads();
  // 1-D structure-factor vectors (mixed path): FP64 weights and twiddles, rounded to FP32
  // once at the end, so that their errors are independent roundings
  if (A.mixed) {
    const int Kx = g.K[0], Ky = g.K[1], Kz = g.K[2];
    const int Kmax = max(Kx, max(Ky, Kz));
    const int total = ns * 3 * Kmax;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int s = (int)__umulhi((unsigned)t, A.m3Kmax);
      const int r = t - s * 3 * Kmax;
      const int ax = (int)__umulhi((unsigned)r, A.mKmax);
      const int k = r - ax * Kmax;
      const int K = g.K[ax];
      if (k >= K) continue;
      const size_t us = (size_t)b * kMaxSoluteSites + s;
      const int grd = sgrd[s][ax];
      const double2* tw = A.twiddle64 + (ax == 0 ? 0 : (ax == 1 ? Kx : Kx + Ky));
      const double* th = a.u_w + (us * 3 + ax) * kMaxSplineOrder;
      const unsigned mk = A.mK[ax];
      double re = 0.0, im = 0.0;
      for (int c = 0; c < P; ++c) {
        int gc = grd - c;  // in (-P, K)
        if (gc < 0) gc += K;
        const unsigned x = (unsigned)(k * gc);  // < K^2 <= 10^6
        const int mm = (int)(x - __umulhi(x, mk) * (unsigned)K);
        const double2 w = tw[mm];
        re = fma(th[c], w.x, re);
        im = fma(th[c], w.y, im);
      }
      a.u_bvec[(us * 3 + ax) * Kmax + k] = make_float2((float)re, (float)im);
    }
  }
  // bounding radius about site 1 (minimum image; FP32, padded to stay conservative)
  __shared__ int rmax_bits;
  if (threadIdx.x == 0) rmax_bits = 0;
  __syncthreads();
  for (int s = 1 + threadIdx.x; s < ns; s += blockDim.x) {
    float r2 = 0.f;
    for (int i = 0; i < 3; ++i) {
      const float h = 0.5f * (float)g.L[i];
      const float d = h - fabsf(h - fabsf((float)(sx[s][i] - sx[0][i])));
      r2 += d * d;
    }
    atomicMax(&rmax_bits, __float_as_int(sqrtf(r2)));  // nonnegative floats order as ints
  }
  __syncthreads();
  if (threadIdx.x == 0) a.u_radius[b] = __int_as_float(rmax_bits) * 1.0001f + 1e-4f;
  // realcal_self (realcal.F90:284-328), fixed-order block reduction
  const bool need_self = (A.self_mode == 1) || (A.self_mode == 2 && b == 0);
  if (need_self && A.bare) {  // realcal_self returns 0 for bare Coulomb (realcal.F90:294)
    if (threadIdx.x == 0) a.u_usreal[b] = 0.0;
    return;
  }
  if (need_self) {
    double acc = 0.0;
    const int npair = ns * ns;  // (is, js) with js >= is; diagonal gives the atom residual
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
      const int is = t / ns, js = t % ns;
      if (js < is) continue;
      const double qi = A.charge[atom0 + is];
      if (js == is) {
        acc += -qi * qi * A.sc.screen / sqrt(kPi);
      } else {
        double d2 = 0.0;
        for (int i = 0; i < 3; ++i) {
          const double h = 0.5 * g.L[i];
          const double d = h - fabs(h - fabs(sx[is][i] - sx[js][i]));
          d2 += d * d;
        }
        const double rst = sqrt(d2);
        acc += -qi * A.charge[atom0 + js] * erf(A.sc.screen * rst) / rst;
      }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) a.u_usreal[b] = red[0];
  }
}

// ---- FP64 path ----------------------------------------------------------------------
struct Spread64Args {
  const double* u_q;
  const double* u_w;
  const int* u_grid;
  const int* u_nsite;
  double* grid;  // [nb][K3][K2][K1]
  int K1, K2, K3, P;
};

// one block per placement; sites in order, the P^3 stencil points of a site in parallel
__global__ void spread64_kernel(Spread64Args A) {
  const int b = blockIdx.x;
  const int ns = A.u_nsite[b];
  const int P = A.P, P3 = P * P * P;
  double* grid = A.grid + (size_t)b * A.K1 * A.K2 * A.K3;
  for (int s = 0; s < ns; ++s) {
    const size_t us = (size_t)b * kMaxSoluteSites + s;
    const int gp = A.u_grid[us];
    const int g1 = gp & 1023, g2 = (gp >> 10) & 1023, g3 = (gp >> 20) & 1023;
    const double chr = A.u_q[us];
    const double* w = A.u_w + us * 3 * kMaxSplineOrder;
    for (int t = threadIdx.x; t < P3; t += blockDim.x) {
      const int cg1 = t % P, cg2 = (t / P) % P, cg3 = t / (P * P);
      int r1 = (g1 - cg1) % A.K1, r2 = (g2 - cg2) % A.K2, r3 = (g3 - cg3) % A.K3;
      if (r1 < 0) r1 += A.K1;
      if (r2 < 0) r2 += A.K2;
      if (r3 < 0) r3 += A.K3;
      const double factor = chr * w[cg1] * w[kMaxSplineOrder + cg2] * w[2 * kMaxSplineOrder + cg3];
      grid[((size_t)r3 * A.K2 + r2) * A.K1 + r1] += factor;
    }
    __syncthreads();
  }
}

struct Infl64Args {
  double2* spec;          // [nb][K3][K2][H]
  const double* engfac;
  double* self_part;      // [nb][nblk]
  int K1, K2, K3, H;
  size_t n;
  int nblk;
};

__global__ void __launch_bounds__(256) influence64_kernel(Infl64Args A) {
  const int b = blockIdx.y;
  double s = 0.0;
  const bool even = (A.K1 % 2) == 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (size_t)gridDim.x * blockDim.x) {
    const int k1 = (int)(i % A.H);
    double2 z = A.spec[(size_t)b * A.n + i];
    const double ef = A.engfac[i];
    const double e = ef * (z.x * z.x + z.y * z.y);
    s += (k1 == 0 || (even && k1 == A.H - 1)) ? 0.5 * e : e;
    A.spec[(size_t)b * A.n + i] = make_double2(ef * z.x, ef * z.y);
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) A.self_part[(size_t)b * A.nblk + blockIdx.x] = red[0];
}

Coef make_coef(int order, double screen) {
  Coef s{};
  s.order = order;
  for (int i = 0; i <= order; ++i) {
    double factor = 1.0;
    for (int k = 1; k <= i; ++k) factor = factor * (double)k;
    for (int k = 1; k <= order - i; ++k) factor = factor * (double)k;
    factor = (double)order / factor;
    if (i % 2 == 1) factor = -factor;
    s.c[i] = factor;
  }
  s.screen = screen;
  return s;
}

}  // namespace

// self-energy partials per placement of the mixed path: one per k2 (the pme_a CTA of
// (k2, placement) writes self_part[b][k2])
int spectrum_partials(const Engine& e) { return e.geom.K[1]; }

cudaError_t launch_place_prep(Engine& e, const BatchArgs& a, const double* sol_xyz, int self_mode, cudaStream_t s) {
  PrepArgs A{};
  A.a = a;
  A.solxyz = sol_xyz;
  A.sitepos = e.d_sitepos;
  A.mbi0 = e.d_mbi0;
  A.charge = e.d_charge;
  A.ljtype = e.d_ljtype;
  A.mol_qmol_all = e.d_qmol_all;
  A.twiddle64 = e.d_twiddle64;
  A.g = e.geom;
  A.sc = make_coef(e.P_order, e.P.screen);
  A.mixed = e.mixed ? 1 : 0;
  A.self_mode = self_mode;
  A.bare = (e.P.cltype == 0) ? 1 : 0;
  A.nummol = e.nummol;
  A.status = e.d_status;
  auto magic = [](unsigned d) { return (unsigned)((0x100000000ull + d - 1) / d); };
  for (int i = 0; i < 3; ++i) A.mK[i] = magic((unsigned)e.geom.K[i]);
  A.mKmax = magic((unsigned)e.Kmax());
  A.m3Kmax = magic(3u * (unsigned)e.Kmax());
  place_prep_kernel<<<a.nb, 256, 0, s>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_spread64(Engine& e, const BatchArgs& a) {
  Spread64Args A{};
  A.u_q = a.u_q;
  A.u_w = a.u_w;
  A.u_grid = a.u_grid;
  A.u_nsite = a.u_nsite;
  A.grid = a.phi64;
  A.K1 = e.geom.K[0];
  A.K2 = e.geom.K[1];
  A.K3 = e.geom.K[2];
  A.P = e.P_order;
  cudaError_t err = cudaMemsetAsync(a.phi64, 0, sizeof(double) * e.grid_real() * a.nb, a.stream);
  if (err != cudaSuccess) return err;
  spread64_kernel<<<a.nb, 128, 0, a.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

int influence64_blocks() { return 152 * 2; }

cudaError_t launch_influence64(Engine& e, const BatchArgs& a) {
  Infl64Args A{};
  A.spec = a.spec64;
  A.engfac = e.d_engfac;
  A.self_part = a.self_part;
  A.K1 = e.geom.K[0];
  A.K2 = e.geom.K[1];
  A.K3 = e.geom.K[2];
  A.H = e.H();
  A.n = e.grid_cplx();
  A.nblk = influence64_blocks();
  dim3 grid(A.nblk, a.nb);
  influence64_kernel<<<grid, 256, 0, a.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
