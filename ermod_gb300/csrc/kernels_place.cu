// kernels_place.cu -- per-placement solute preparation and the PME solute potential.
//
//   place_prep    solute sites of every placement in a batch: wrapped FP64 and
//                 fixed-point coordinates, calc_spline_molecule (recpcal.F90:408-442),
//                 realcal_self (realcal.F90:284-328, FP64) and, for the mixed path,
//                 the 1-D structure-factor vectors
//                     b_{s,a}(k) = sum_c theta_{s,a,c} exp(-2 pi i k (g_{s,a} - c) / K_a);
//   spectrum      mixed path: the spread charge grid of recpcal_prepare_solute
//                 (recpcal.F90:357-373) followed by its R2C transform (recpcal.F90:377)
//                 equals S(k) = sum_s q_s b_{s,1}(k1) b_{s,2}(k2) b_{s,3}(k3) exactly; this
//                 kernel evaluates S on the half-complex grid directly (FP32), multiplies
//                 by engfac (recpcal.F90:398) and reduces the self energy
//                 (recpcal.F90:385-394) with float-float compensation into FP64 partials.
//                 It replaces a K^3 zero-fill, a scattered spread and a forward FFT by a
//                 compute-bound pass that writes only the half spectrum.
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
  const float2* twiddle;       // [K1+K2+K3]
  FrameGeom g;
  Coef sc;
  int mixed;
  int self_mode;  // 0: none, 1: all placements, 2: only placement 0 of the batch
  int nummol;
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
    if (is_atom1) {  // atom 1 itself takes the first-pass x shift of its own x
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
      for (int spi = 0; spi < P; ++spi)
        a.u_w[(us * 3 + kk) * kMaxSplineOrder + spi] = spline_value(A.sc, f2 - (double)(rci[kk] - spi));
    }
    a.u_grid[us] = rci[0] | (rci[1] << kGridBits) | (rci[2] << (2 * kGridBits));
  }
  if (threadIdx.x == 0) {
    a.u_nsite[b] = ns;
    a.u_qmol[b] = A.mol_qmol_all[mol];
  }
  __syncthreads();
  // 1-D structure-factor vectors (mixed path)
  if (A.mixed) {
    const int Kx = g.K[0], Ky = g.K[1], Kz = g.K[2];
    const int Kmax = max(Kx, max(Ky, Kz));
    const int total = ns * 3 * Kmax;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int k = t % Kmax;
      const int ax = (t / Kmax) % 3;
      const int s = t / (3 * Kmax);
      const int K = g.K[ax];
      if (k >= K) continue;
      const size_t us = (size_t)b * kMaxSoluteSites + s;
      const int grd = (a.u_grid[us] >> (ax * kGridBits)) & ((1 << kGridBits) - 1);
      const float2* tw = A.twiddle + (ax == 0 ? 0 : (ax == 1 ? Kx : Kx + Ky));
      float re = 0.f, im = 0.f;
      for (int c = 0; c < P; ++c) {
        const float th = (float)a.u_w[(us * 3 + ax) * kMaxSplineOrder + c];
        int mm = (k * (grd - c)) % K;  // |k (grd - c)| < 1000 * 1008 fits in int
        if (mm < 0) mm += K;
        const float2 w = tw[mm];
        re = fmaf(th, w.x, re);
        im = fmaf(th, w.y, im);
      }
      a.u_bvec[(us * 3 + ax) * Kmax + k] = make_float2(re, im);
    }
  }
  // bounding radius about site 1 (minimum image)
  if (threadIdx.x == 0) {
    double rmax = 0.0;
    for (int s = 1; s < ns; ++s) {
      double r2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double h = 0.5 * g.L[i];
        const double d = h - fabs(h - fabs(sx[s][i] - sx[0][i]));
        r2 += d * d;
      }
      rmax = fmax(rmax, sqrt(r2));
    }
    a.u_radius[b] = (float)rmax * 1.0001f + 1e-4f;
  }
  // realcal_self (realcal.F90:284-328), fixed-order block reduction
  const bool need_self = (A.self_mode == 1) || (A.self_mode == 2 && b == 0);
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

// float-float accumulation (Dekker/Knuth TwoSum)
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff ff_add(ff a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b - bb);
  const float lo = a.lo + err;
  const float hi = s + lo;
  return ff{hi, lo - (hi - s)};
}
__device__ __forceinline__ ff ff_add2(ff a, ff b) {
  ff r = ff_add(a, b.hi);
  return ff_add(r, b.lo);
}

constexpr int kSpecThreads = 256;
constexpr int kSpecChunk = 32;  // solute sites staged in shared memory at once
constexpr int kR1 = 4, kR2 = 4;  // register micro-tile: 4 k1 x 4 k2 points per thread

struct SpecArgs {
  const float2* bvec;     // [nb][S][3][Kmax]
  const double* u_q;      // [nb][S]
  const int* u_nsite;
  const float* engfac;    // [K3][K2][H]
  float2* spec;           // [nb][K3][K2][H]
  double* self_part;      // [nb][K3]
  int K1, K2, K3, H, Kmax;
};

// grid: (K3, nb); one CTA computes the (k1, k2) plane of one k3 for one placement:
//   Q(k1,k2,k3) = sum_s [q_s b3_s(k3) b2_s(k2)] b1_s(k1)
// as a sum of rank-1 updates over register micro-tiles of 4 x 4 points.
__global__ void __launch_bounds__(kSpecThreads) spectrum_kernel(SpecArgs A) {
  extern __shared__ float2 smem_spec[];
  float2* sd = smem_spec;                           // [kSpecChunk][K2]
  float2* sb = smem_spec + (size_t)kSpecChunk * A.K2;  // [kSpecChunk][H padded to 4]
  const int k3 = blockIdx.x, b = blockIdx.y;
  const int ns = A.u_nsite[b];
  const int TX = (A.H + kR1 - 1) / kR1, TY = (A.K2 + kR2 - 1) / kR2;
  const int Hp = TX * kR1;
  const int ntiles = TX * TY;
  const float2* bv = A.bvec + (size_t)b * kMaxSoluteSites * 3 * A.Kmax;
  float2* spec = A.spec + (size_t)b * A.K3 * A.K2 * A.H + (size_t)k3 * A.K2 * A.H;
  const float* ef = A.engfac + (size_t)k3 * A.K2 * A.H;
  const bool even = (A.K1 % 2) == 0;
  ff self{0.f, 0.f};
  for (int s0 = 0; s0 < ns; s0 += kSpecChunk) {
    const int nsc = min(kSpecChunk, ns - s0);
    const bool first = (s0 == 0), last = (s0 + nsc >= ns);
    __syncthreads();
    for (int t = threadIdx.x; t < nsc * A.K2; t += blockDim.x) {
      const int sl = t / A.K2, k2 = t % A.K2;
      const size_t us = (size_t)(s0 + sl);
      const float q = (float)A.u_q[(size_t)b * kMaxSoluteSites + us];
      const float2 b3 = bv[(us * 3 + 2) * A.Kmax + k3];
      const float2 b2 = bv[(us * 3 + 1) * A.Kmax + k2];
      const float2 c3 = make_float2(q * b3.x, q * b3.y);
      sd[sl * A.K2 + k2] = make_float2(c3.x * b2.x - c3.y * b2.y, c3.x * b2.y + c3.y * b2.x);
    }
    for (int t = threadIdx.x; t < nsc * Hp; t += blockDim.x) {
      const int sl = t / Hp, k1 = t % Hp;
      sb[sl * Hp + k1] = (k1 < A.H) ? bv[((size_t)(s0 + sl) * 3 + 0) * A.Kmax + k1] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int mt = threadIdx.x; mt < ntiles; mt += blockDim.x) {
      const int tx = mt % TX, ty = mt / TX;
      const int k1a = tx * kR1, k2a = ty * kR2;
      float2 acc[kR2][kR1];
#pragma unroll
      for (int j = 0; j < kR2; ++j)
#pragma unroll
        for (int i = 0; i < kR1; ++i) acc[j][i] = make_float2(0.f, 0.f);
      for (int sl = 0; sl < nsc; ++sl) {
        float2 d[kR2], e[kR1];
#pragma unroll
        for (int j = 0; j < kR2; ++j) d[j] = (k2a + j < A.K2) ? sd[sl * A.K2 + k2a + j] : make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < kR1; ++i) e[i] = sb[sl * Hp + k1a + i];
#pragma unroll
        for (int j = 0; j < kR2; ++j)
#pragma unroll
          for (int i = 0; i < kR1; ++i) {
            acc[j][i].x = fmaf(d[j].x, e[i].x, fmaf(-d[j].y, e[i].y, acc[j][i].x));
            acc[j][i].y = fmaf(d[j].x, e[i].y, fmaf(d[j].y, e[i].x, acc[j][i].y));
          }
      }
#pragma unroll
      for (int j = 0; j < kR2; ++j) {
        const int k2 = k2a + j;
        if (k2 >= A.K2) continue;
#pragma unroll
        for (int i = 0; i < kR1; ++i) {
          const int k1 = k1a + i;
          if (k1 >= A.H) continue;
          const size_t gi = (size_t)k2 * A.H + k1;
          float2 q = acc[j][i];
          if (!first) {  // earlier site chunks left the partial sum in the output
            const float2 prev = spec[gi];
            q.x += prev.x;
            q.y += prev.y;
          }
          if (last) {
            const float f = ef[gi];
            const float wgt = (k1 == 0 || (even && k1 == A.H - 1)) ? 0.5f : 1.f;
            self = ff_add(self, wgt * f * (q.x * q.x + q.y * q.y));
            q = make_float2(f * q.x, f * q.y);
          }
          spec[gi] = q;
        }
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    ff o{__shfl_down_sync(0xffffffffu, self.hi, off), __shfl_down_sync(0xffffffffu, self.lo, off)};
    self = ff_add2(self, o);
  }
  __shared__ double wsum[kSpecThreads / 32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = (double)self.hi + (double)self.lo;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSpecThreads / 32; ++w) t += wsum[w];
    A.self_part[(size_t)b * A.K3 + k3] = t;
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

int spectrum_partials(const Engine& e) { return e.geom.K[2]; }

cudaError_t launch_place_prep(Engine& e, const BatchArgs& a, const double* sol_xyz, int self_mode) {
  PrepArgs A{};
  A.a = a;
  A.solxyz = sol_xyz;
  A.sitepos = e.d_sitepos;
  A.mbi0 = e.d_mbi0;
  A.charge = e.d_charge;
  A.ljtype = e.d_ljtype;
  A.mol_qmol_all = e.d_qmol_all;
  A.twiddle = e.d_twiddle;
  A.g = e.geom;
  A.sc = make_coef(e.P_order, e.P.screen);
  A.mixed = e.mixed ? 1 : 0;
  A.self_mode = self_mode;
  A.nummol = e.nummol;
  A.status = e.d_status;
  place_prep_kernel<<<a.nb, 256, 0, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_spectrum(Engine& e, const BatchArgs& a) {
  SpecArgs A{};
  A.bvec = a.u_bvec;
  A.u_q = a.u_q;
  A.u_nsite = a.u_nsite;
  A.engfac = e.d_engfac_f;
  A.spec = a.spec;
  A.self_part = a.self_part;
  A.K1 = e.geom.K[0];
  A.K2 = e.geom.K[1];
  A.K3 = e.geom.K[2];
  A.H = e.H();
  A.Kmax = e.Kmax();
  const int Hp = ((A.H + kR1 - 1) / kR1) * kR1;
  const size_t smem = sizeof(float2) * (size_t)kSpecChunk * (A.K2 + Hp);
  static size_t attr = 0;
  if (attr < smem) {
    cudaError_t err = cudaFuncSetAttribute(spectrum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    attr = smem;
  }
  dim3 grid(A.K3, a.nb);
  spectrum_kernel<<<grid, kSpecThreads, smem, e.stream>>>(A);
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
  cudaError_t err = cudaMemsetAsync(a.phi64, 0, sizeof(double) * e.grid_real() * a.nb, e.stream);
  if (err != cudaSuccess) return err;
  spread64_kernel<<<a.nb, 128, 0, e.stream>>>(A);
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
  influence64_kernel<<<grid, 256, 0, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
