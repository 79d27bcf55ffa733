// kernels_frame.cu -- once-per-frame preparation (the engconst prologue).
//
//   frame_wrap      realcal_prepare + normalize_periodic (realcal.F90:137-146, 789-885)
//                   for every atom, FP64, the reference's two wrap passes;
//   frame_sort      spatial (Morton) order of the physical molecules by the ~4 A cell of
//                   their first site, so that a CTA's molecules are compact in space
//                   (coherent near-field branches, PME-grid reuse in L1);
//   frame_sites     per physical site in slot order: fixed-point coordinates, LJ type,
//                   charge and the B-spline data of calc_spline_molecule
//                   (recpcal.F90:408-442) -- replaces recpcal_prepare_solvent
//                   (engproc.F90:378-382) and the per-placement blockify/sort_block
//                   rebuild of the reference (realcal.F90:439-525);
//   greenfunc       recpcal_spline_greenfunc (recpcal.F90:111-152), FP64; for PPPM
//                   (cltype 3) recpcal_pppm_greenfunc (recpcal.F90:205-319).
// All of these are HBM-streaming kernels over O(numatm) or O(K^3) elements.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cmath>
#include <cstring>

#include "bestfit.cuh"
#include "engine.cuh"

namespace ermod {

namespace {

struct SplineCoef {
  double c[kMaxSplineOrder + 1];
  int order;
};

SplineCoef make_coef(int order) {  // spline_init, spline.F90:26-44
  SplineCoef s{};
  s.order = order;
  for (int i = 0; i <= order; ++i) {
    double factor = 1.0;
    for (int k = 1; k <= i; ++k) factor = factor * (double)k;
    for (int k = 1; k <= order - i; ++k) factor = factor * (double)k;
    factor = (double)order / factor;
    if (i % 2 == 1) factor = -factor;
    s.c[i] = factor;
  }
  return s;
}

__host__ __device__ __forceinline__ double ipow(double x, int e) {
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

// spline_value (spline.F90:47-59)
__device__ __forceinline__ double spline_value(const SplineCoef& s, double rst) {
  double f = 0.0;
  if ((rst > 0.0) && (rst < (double)s.order)) {
    const int k = (int)rst;
    for (int i = 0; i <= k; ++i) f = f + s.c[i] * ipow(rst - (double)i, s.order - 1);
  }
  return f;
}

// normalize_periodic for a cuboid cell, atom a (0-based); mirrors both passes.
__device__ __forceinline__ void wrap_atom(const double* __restrict__ pos, int a, const FrameGeom& g, double out[3]) {
  double x[3];
  for (int i = 0; i < 3; ++i) {
    const double v = pos[3 * (size_t)a + i];
    x[i] = v - g.L[i] * floor(g.invL[i] * v);
  }
  // second pass: y by the second cell vector, x by atom 1's current x (realcal.F90:878-883)
  x[1] = x[1] - g.L[1] * floor(g.invL[1] * x[1]);
  const double x0 = pos[0] - g.L[0] * floor(g.invL[0] * pos[0]);
  const double f0 = floor(g.invL[0] * x0);
  if (a == 0) {
    x[0] = x[0] - g.L[0] * f0;
  } else {
    const double x0b = x0 - g.L[0] * f0;
    x[0] = x[0] - g.L[0] * floor(g.invL[0] * x0b);
  }
  out[0] = x[0];
  out[1] = x[1];
  out[2] = x[2];
}

__global__ void frame_wrap_kernel(const double* __restrict__ pos, int numatm, FrameGeom g, double* __restrict__ out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= numatm) return;
  double w[3];
  if (g.periodic) {
    wrap_atom(pos, a, g, w);
  } else {  // non-periodic: realcal_prepare copies the coordinates as they are
    for (int i = 0; i < 3; ++i) w[i] = pos[3 * (size_t)a + i];
  }
  out[3 * (size_t)a + 0] = w[0];
  out[3 * (size_t)a + 1] = w[1];
  out[3 * (size_t)a + 2] = w[2];
}

__device__ __forceinline__ unsigned int spread3(unsigned int v) {
  v &= 0x3ff;
  v = (v | (v << 16)) & 0x030000ff;
  v = (v | (v << 8)) & 0x0300f00f;
  v = (v | (v << 4)) & 0x030c30c3;
  v = (v | (v << 2)) & 0x09249249;
  return v;
}

__global__ void frame_key_kernel(const double* __restrict__ wrapped, const int* __restrict__ mol_atom0, int slvmax,
                                 FrameGeom g, int3 ncell, unsigned int* __restrict__ key, int* __restrict__ val) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= slvmax) return;
  const int a = mol_atom0[k];
  int c[3];
  const int n[3] = {ncell.x, ncell.y, ncell.z};
  for (int i = 0; i < 3; ++i) {
    // non-periodic coordinates lie in (-L/2, L/2) of the virtual cube
    const double f = wrapped[3 * (size_t)a + i] * g.invL[i] + (g.periodic ? 0.0 : 0.5);
    int ci = (int)(f * (double)n[i]);
    c[i] = min(max(ci, 0), n[i] - 1);
  }
  key[k] = spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
  val[k] = k;
}

__global__ void frame_slot_kernel(const int* __restrict__ slot_mol, const int* __restrict__ mol_nsite,
                                  const int* __restrict__ mol_species, const double* __restrict__ mol_qmol,
                                  int slvmax, int* __restrict__ slot_nsite, int* __restrict__ slot_species,
                                  double* __restrict__ slot_qmol) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= slvmax) return;
  const int k = slot_mol[m];
  slot_nsite[m] = mol_nsite[k];
  slot_species[m] = mol_species[k];
  slot_qmol[m] = mol_qmol[k];
}

struct SiteArgs {
  const double* pos;      // raw sitepos
  const double* wrapped;  // normalised sitepos
  const int* slot_mol;
  const int* slot_site;
  const int* mol_atom0;
  const int* mol_nsite;
  const double* charge;
  const int* ljtype;
  int slvmax;
  int mixed;
  FrameGeom g;
  SplineCoef sc;
  int4* site_pos;
  float4* site_rec;
  int* site_grid;
  double* site_x;
  double* site_w;
  double* site_q;
  float* frame_scal;
};

// one thread per slot (molecule): its sites
__global__ void frame_sites_kernel(SiteArgs A) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  double rmax = 0.0;
  if (m < A.slvmax) {  // (no early return: the warp's maximum below takes every lane)
    const int k = A.slot_mol[m];
    const int a0 = A.mol_atom0[k];
    const int ns = A.mol_nsite[k];
    const int s0 = A.slot_site[m];
    const FrameGeom& g = A.g;
    const int P = A.sc.order;
    double w0[3] = {A.wrapped[3 * (size_t)a0], A.wrapped[3 * (size_t)a0 + 1], A.wrapped[3 * (size_t)a0 + 2]};
    for (int s = 0; s < ns; ++s) {
      const int a = a0 + s;
      const int idx = s0 + s;
      double w[3] = {A.wrapped[3 * (size_t)a], A.wrapped[3 * (size_t)a + 1], A.wrapped[3 * (size_t)a + 2]};
      // radius about the first site (minimum image)
      double r2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double h = 0.5 * g.L[i];
        const double d = h - fabs(h - fabs(w[i] - w0[i]));
        r2 += d * d;
      }
      rmax = fmax(rmax, sqrt(r2));
      // calc_spline_molecule (recpcal.F90:408-442) on the raw coordinates
      const double xst[3] = {A.pos[3 * (size_t)a], A.pos[3 * (size_t)a + 1], A.pos[3 * (size_t)a + 2]};
      int rci[3];
      double tfrac[3];
      for (int kk = 0; kk < 3; ++kk) {
        double factor = g.invcl[kk + 0] * xst[0] + g.invcl[kk + 3] * xst[1] + g.invcl[kk + 6] * xst[2];
        factor = factor - floor(factor);
        const double f2 = factor * (double)g.K[kk];
        rci[kk] = (int)f2;
        tfrac[kk] = f2 - (double)rci[kk];
        if (!A.mixed) {
          for (int spi = 0; spi < P; ++spi)
            A.site_w[((size_t)idx * 3 + kk) * P + spi] = spline_value(A.sc, f2 - (double)(rci[kk] - spi));
        }
      }
      A.site_grid[idx] = rci[0] | (rci[1] << kGridBits) | (rci[2] << (2 * kGridBits));
      const double q = A.charge[a];
      // FP64 wrapped coordinates and charge: the FP64 path's pair terms, and the mixed
      // path's FP64 terms of close pairs
      A.site_x[3 * (size_t)idx + 0] = w[0];
      A.site_x[3 * (size_t)idx + 1] = w[1];
      A.site_x[3 * (size_t)idx + 2] = w[2];
      A.site_q[idx] = q;
      if (A.mixed) {
        unsigned int X[3];
        for (int i = 0; i < 3; ++i) {
          const double u = w[i] * g.invL[i] * 4294967296.0;
          X[i] = (unsigned int)(unsigned long long)llrint(u);
        }
        A.site_pos[idx] = make_int4((int)X[0], (int)X[1], (int)X[2], A.ljtype[a]);
        A.site_rec[idx] = make_float4((float)tfrac[0], (float)tfrac[1], (float)tfrac[2], (float)q);
      } else {
        A.site_pos[idx] = make_int4(0, 0, 0, A.ljtype[a]);
      }
    }
  }
  // the largest molecule radius: a warp maximum first, then one atomic per warp on this
  // one address instead of one per molecule
  float r = (m < A.slvmax) ? (float)rmax * 1.0001f + 1e-4f : 0.f;
  for (int off = 16; off > 0; off >>= 1) r = fmaxf(r, __shfl_xor_sync(0xffffffffu, r, off));
  if ((threadIdx.x & 31) == 0) atomicMax((int*)&A.frame_scal[0], __float_as_int(r));
}

// brick of every site: the kBrickX x kBrickY x kBrickZ block of PME grid points holding its
// stencil base point
__global__ void brick_key_kernel(const int* __restrict__ site_grid, int nsite, int K1, int K2, int K3, int nbx,
                                 int nby, unsigned int* __restrict__ key, int* __restrict__ val,
                                 int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsite) return;
  const int gp = site_grid[i];
  int g1 = gp & 1023, g2 = (gp >> 10) & 1023, g3 = (gp >> 20) & 1023;
  if (g1 >= K1) g1 -= K1;
  if (g2 >= K2) g2 -= K2;
  if (g3 >= K3) g3 -= K3;
  const unsigned int bk = (unsigned int)(((g3 / kBrickZ) * nby + (g2 / kBrickY)) * nbx + (g1 / kBrickX));
  key[i] = bk;
  val[i] = i;
  atomicAdd(&count[bk], 1);
}

// the FP32 copy of engfac keeps rows of H points padded to a multiple of 4 (zeros)
__device__ __forceinline__ size_t padded_row_index(size_t i, int H) {
  return (i / H) * (size_t)(((H + 3) / 4) * 4) + i % H;
}

// recpcal_spline_greenfunc (recpcal.F90:111-152)
__global__ void greenfunc_kernel(FrameGeom g, int order, const double* __restrict__ splfc, double screen,
                                 double* __restrict__ engfac, float* __restrict__ engfac_f) {
  const int H = g.K[0] / 2 + 1;
  const size_t n = (size_t)H * g.K[1] * g.K[2];
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int rc1 = (int)(i % H);
  const int rc2 = (int)((i / H) % g.K[1]);
  const int rc3 = (int)(i / ((size_t)H * g.K[1]));
  double factor = 0.0;
  if (!(rc1 == 0 && rc2 == 0 && rc3 == 0)) {
    const int rc[3] = {rc1, rc2, rc3};
    double inm[3];
    bool zero = false;
    for (int m = 0; m < 3; ++m) {
      const int rcimax = g.K[m];
      if ((order % 2 == 1) && (2 * abs(rc[m]) == rcimax)) zero = true;
      inm[m] = (rc[m] <= rcimax / 2) ? (double)rc[m] : (double)(rc[m] - rcimax);
    }
    if (!zero) {
      double xst[3];
      for (int m = 0; m < 3; ++m)
        xst[m] = g.invcl[0 + 3 * m] * inm[0] + g.invcl[1 + 3 * m] * inm[1] + g.invcl[2 + 3 * m] * inm[2];
      double rtp2 = xst[0] * xst[0] + xst[1] * xst[1] + xst[2] * xst[2];
      const double chr = (kPi * kPi) * rtp2 / (screen * screen);
      factor = exp(-chr) / rtp2 / kPi / g.volume;
      rtp2 = splfc[rc1] * splfc[g.K[0] + rc2] * splfc[g.K[0] + g.K[1] + rc3];
      factor = factor / rtp2;
    }
  }
  engfac[i] = factor;
  engfac_f[padded_row_index(i, H)] = (float)factor;
}

// recpcal_pppm_greenfunc (recpcal.F90:205-319): the optimal influence function of PPPM,
// summed over the aliases mx, my, mz in [-m_max, m_max] (m_max from cell . LAMMPS'
// estimate); mN(3) = mz * ms2max as the reference writes it.
struct PppmArgs {
  FrameGeom g;
  int order;
  int mmax[3];
  double screen;
  double gf_b[kMaxSplineOrder + 1];  // calc_gfb_pppm, 0-based
};

__device__ __forceinline__ double ipow_int(double x, int e) {
  double r = 1.0;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

__global__ void pppm_greenfunc_kernel(PppmArgs A, double* __restrict__ engfac, float* __restrict__ engfac_f) {
  const FrameGeom& g = A.g;
  const int H = g.K[0] / 2 + 1;
  const size_t n = (size_t)H * g.K[1] * g.K[2];
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int rc[3] = {(int)(i % H), (int)((i / H) % g.K[1]), (int)(i / ((size_t)H * g.K[1]))};
  double factor = 0.0;
  if (!(rc[0] == 0 && rc[1] == 0 && rc[2] == 0)) {
    double inm[3], s2[3], k[3];
    for (int a = 0; a < 3; ++a) {
      inm[a] = (rc[a] <= g.K[a] / 2) ? (double)rc[a] : (double)(rc[a] - g.K[a]);
      const double sn = sin(kPi * inm[a] / g.K[a]);
      s2[a] = sn * sn;
    }
    for (int a = 0; a < 3; ++a)
      k[a] = 2 * kPi * (g.invcl[0 + 3 * a] * inm[0] + g.invcl[1 + 3 * a] * inm[1] + g.invcl[2 + 3 * a] * inm[2]);
    const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    if (k2 > 0.0) {
      double sum = 0.0;
      for (int mx = -A.mmax[0]; mx <= A.mmax[0]; ++mx) {
        double t = kPi * (inm[0] / g.K[0] + mx);
        const double u1 = (t == 0.0) ? 1.0 : ipow_int(sin(t) / t, 2 * A.order);
        for (int my = -A.mmax[1]; my <= A.mmax[1]; ++my) {
          t = kPi * (inm[1] / g.K[1] + my);
          const double u2 = (t == 0.0) ? 1.0 : ipow_int(sin(t) / t, 2 * A.order);
          for (int mz = -A.mmax[2]; mz <= A.mmax[2]; ++mz) {
            t = kPi * (inm[2] / g.K[2] + mz);
            const double u3 = (t == 0.0) ? 1.0 : ipow_int(sin(t) / t, 2 * A.order);
            const double mN[3] = {(double)(mx * g.K[0]), (double)(my * g.K[1]), (double)(mz * g.K[1])};
            double km[3], gam = 1.0;
            for (int a = 0; a < 3; ++a) {
              km[a] = k[a] + 2 * kPi * (g.invcl[0 + 3 * a] * mN[0] + g.invcl[1 + 3 * a] * mN[1] +
                                        g.invcl[2 + 3 * a] * mN[2]);
              const double q = km[a] / A.screen;
              gam *= exp(-0.25 * (q * q));
            }
            const double kkm = k[0] * km[0] + k[1] * km[1] + k[2] * km[2];
            const double km2 = km[0] * km[0] + km[1] * km[1] + km[2] * km[2];
            sum = sum + kkm * gam * (u1 * u2 * u3) / km2;
          }
        }
      }
      double den[3] = {0.0, 0.0, 0.0};  // gf_denom
      for (int l = A.order - 1; l >= 0; --l)
        for (int a = 0; a < 3; ++a) den[a] = A.gf_b[l] + den[a] * s2[a];
      const double d = den[0] * den[1] * den[2];
      factor = sum * 4.0 * kPi / (k2 * (d * d)) / g.volume;
    }
  }
  engfac[i] = factor;
  engfac_f[padded_row_index(i, H)] = (float)factor;
}

inline int nblk(size_t n, int t) { return (int)((n + t - 1) / t); }

// largest |x| of n doubles (non-finite values give a non-finite result): one block, the
// bit patterns of nonnegative doubles order as unsigned integers, NaN above infinity
__global__ void max_abs_kernel(const double* __restrict__ x, size_t n, unsigned long long* __restrict__ out) {
  unsigned long long m = 0ull;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(x[i]));
    m = b > m ? b : m;
  }
  atomicMax(out, m);
}

// device API, at the start of a call: an error left by an earlier call moves to
// first_key, and err_key keeps it with placement index 0 so that every batch of this
// call is skipped by the accumulation (its skip test compares the placement index)
__global__ void carry_status_kernel(DevStatus* s) {
  const unsigned long long k = s->err_key;
  if (k != kNoError) {
    if (s->first_key == kNoError) s->first_key = k;
    s->err_key = s->first_key & ((1ull << 36) - 1);
  }
}

}  // namespace

cudaError_t launch_carry_status(Engine& e) {
  carry_status_kernel<<<1, 1, 0, e.stream>>>(e.d_status);
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_max_abs(Engine& e, const double* x_d, size_t n, double* host_out) {
  unsigned long long* d = reinterpret_cast<unsigned long long*>(e.d_frame_scal + 2);  // 8-byte aligned scratch
  cudaError_t err = cudaMemsetAsync(d, 0, sizeof(unsigned long long), e.stream);
  if (err != cudaSuccess) return err;
  max_abs_kernel<<<1, 1024, 0, e.stream>>>(x_d, n, d);
  e.count_launch();
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  unsigned long long h = 0ull;
  if ((err = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, e.stream)) != cudaSuccess) return err;
  if ((err = cudaStreamSynchronize(e.stream)) != cudaSuccess) return err;
  std::memcpy(host_out, &h, sizeof(h));
  return cudaSuccess;
}

cudaError_t launch_frame_wrap(Engine& e) {
  frame_wrap_kernel<<<nblk(e.numatm, 256), 256, 0, e.stream>>>(e.d_sitepos, e.numatm, e.geom, e.d_wrapped);
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_frame_sort(Engine& e) {
  int3 nc;
  nc.x = std::max(1, std::min(1024, (int)(e.geom.L[0] / 4.0)));
  nc.y = std::max(1, std::min(1024, (int)(e.geom.L[1] / 4.0)));
  nc.z = std::max(1, std::min(1024, (int)(e.geom.L[2] / 4.0)));
  frame_key_kernel<<<nblk(e.slvmax, 256), 256, 0, e.stream>>>(e.d_wrapped, e.d_mol_atom0, e.slvmax, e.geom, nc,
                                                             e.d_sort_key, e.d_sort_val);
  e.count_launch();
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  size_t bytes = e.cub_tmp_bytes;
  err = cub::DeviceRadixSort::SortPairs(e.d_cub_tmp, bytes, e.d_sort_key, e.d_sort_key_alt, e.d_sort_val,
                                        e.d_slot_mol, e.slvmax, 0, 30, e.stream);
  if (err != cudaSuccess) return err;
  frame_slot_kernel<<<nblk(e.slvmax, 256), 256, 0, e.stream>>>(e.d_slot_mol, e.d_mol_nsite, e.d_mol_species,
                                                              e.d_mol_qmol, e.slvmax, e.d_sort_val_alt,
                                                              e.d_slot_species, e.d_slot_qmol);
  e.count_launch();
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  bytes = e.cub_tmp_bytes;
  // slot_site = exclusive scan of slot_nsite, with slot_site[slvmax] = total
  err = cub::DeviceScan::ExclusiveSum(e.d_cub_tmp, bytes, e.d_sort_val_alt, e.d_slot_site, e.slvmax + 1, e.stream);
  return err;
}

cudaError_t launch_frame_bricks(Engine& e) {
  cudaError_t err = cudaMemsetAsync(e.d_brick_count, 0, sizeof(int) * (e.nbricks + 1), e.stream);
  if (err != cudaSuccess) return err;
  brick_key_kernel<<<nblk(e.nsite_phys, 256), 256, 0, e.stream>>>(e.d_site_grid, e.nsite_phys, e.geom.K[0],
                                                                   e.geom.K[1], e.geom.K[2], e.nbrick[0],
                                                                   e.nbrick[1], e.d_brick_key, e.d_brick_val,
                                                                   e.d_brick_count);
  e.count_launch();
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  int bits = 1;
  while ((1 << bits) < e.nbricks + 1) ++bits;
  size_t bytes = e.cub_tmp_bytes;
  err = cub::DeviceRadixSort::SortPairs(e.d_cub_tmp, bytes, e.d_brick_key, e.d_brick_key_alt, e.d_brick_val,
                                        e.d_brick_site, e.nsite_phys, 0, bits, e.stream);
  if (err != cudaSuccess) return err;
  bytes = e.cub_tmp_bytes;
  return cub::DeviceScan::ExclusiveSum(e.d_cub_tmp, bytes, e.d_brick_count, e.d_brick_start, e.nbricks + 1,
                                       e.stream);
}

size_t frame_cub_bytes(int n) {
  size_t a = 0, b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, a, (unsigned int*)nullptr, (unsigned int*)nullptr, (int*)nullptr,
                                  (int*)nullptr, n, 0, 30, (cudaStream_t)0);
  cub::DeviceScan::ExclusiveSum(nullptr, b, (int*)nullptr, (int*)nullptr, n + 1, (cudaStream_t)0);
  return std::max(a, b);
}

size_t brick_cub_bytes(int nsite, int nbricks) {
  size_t a = 0, b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, a, (unsigned int*)nullptr, (unsigned int*)nullptr, (int*)nullptr,
                                  (int*)nullptr, nsite, 0, 32, (cudaStream_t)0);
  cub::DeviceScan::ExclusiveSum(nullptr, b, (int*)nullptr, (int*)nullptr, nbricks + 1, (cudaStream_t)0);
  return std::max(a, b);
}

cudaError_t launch_frame_sites(Engine& e) {
  cudaError_t err = cudaMemsetAsync(e.d_frame_scal, 0, sizeof(float) * 4, e.stream);
  if (err != cudaSuccess) return err;
  SiteArgs A{};
  A.pos = e.d_sitepos;
  A.wrapped = e.d_wrapped;
  A.slot_mol = e.d_slot_mol;
  A.slot_site = e.d_slot_site;
  A.mol_atom0 = e.d_mol_atom0;
  A.mol_nsite = e.d_mol_nsite;
  A.charge = e.d_charge;
  A.ljtype = e.d_ljtype;
  A.slvmax = e.slvmax;
  A.mixed = e.mixed ? 1 : 0;
  A.g = e.geom;
  A.sc = make_coef(e.P_order);
  A.site_pos = e.d_site_pos;
  A.site_rec = e.d_site_rec;
  A.site_grid = e.d_site_grid;
  A.site_x = e.d_site_x;
  A.site_w = e.d_site_w;
  A.site_q = e.d_site_q;
  A.frame_scal = e.d_frame_scal;
  // a thread per molecule, its FP64 arithmetic on GB300's narrow FP64 pipe: small systems
  // take warp-sized blocks, so that their molecules spread over many SMs instead of a few
  const int sm2 = 2 * e.num_sm;  // two blocks per SM
  const int nthr = std::min(128, std::max(32, 32 * ((e.slvmax + sm2 * 32 - 1) / (sm2 * 32))));
  frame_sites_kernel<<<nblk(e.slvmax, nthr), nthr, 0, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

// calc_gfb_pppm (recpcal.F90:170-188), including its use of the inner loop variable
// after the loop (l = 0)
static void pppm_gfb(int p, double* out) {
  std::vector<double> b(p + 2, 0.0);  // 1-based
  b[1] = 1.0;
  for (int m = 1; m <= p - 1; ++m) {
    for (int l = m; l >= 1; --l)
      b[l + 1] = 4.0 * (b[l + 1] * (double)(l - m) * ((double)(l - m) - 0.5) - b[l] * (double)((l - m - 1) * (l - m - 1)));
    const int l = 0;
    b[1] = 4.0 * (b[1] * (double)(l - m) * ((double)(l - m) - 0.5));
  }
  double fact = 1.0;
  for (int i = 1; i <= 2 * p - 1; ++i) fact *= (double)i;
  const double gaminv = 1.0 / fact;
  for (int m = 1; m <= p; ++m) out[m - 1] = b[m] * gaminv;
}

cudaError_t launch_greenfunc(Engine& e) {
  if (e.P.cltype == 3) {
    PppmArgs A{};
    A.g = e.geom;
    A.order = e.P_order;
    A.screen = e.P.screen;
    pppm_gfb(e.P_order, A.gf_b);
    const double eps_hoc = 0.0000001;  // LAMMPS' value, recpcal.F90:213
    double mmax[3];
    for (int a = 0; a < 3; ++a) mmax[a] = e.P.screen / (kPi * e.geom.K[a]) * std::pow(-std::log(eps_hoc), 0.25);
    for (int j = 0; j < 3; ++j)  // int(dot_product(cell(:, j), m_max(:)))
      A.mmax[j] = (int)(e.cell[3 * j] * mmax[0] + e.cell[3 * j + 1] * mmax[1] + e.cell[3 * j + 2] * mmax[2]);
    const size_t n = e.grid_cplx();
    pppm_greenfunc_kernel<<<nblk(n, 128), 128, 0, e.stream>>>(A, e.d_engfac, e.d_engfac_f);
    e.count_launch();
    return cudaGetLastError();
  }
  const size_t n = e.grid_cplx();
  greenfunc_kernel<<<nblk(n, 256), 256, 0, e.stream>>>(e.geom, e.P_order, e.d_splfc, e.P.screen, e.d_engfac,
                                                       e.d_engfac_f);
  e.count_launch();
  return cudaGetLastError();
}

// host-side spline_value for the splfc tables (init_spline_axis, recpcal.F90:87-109)
double host_spline_value(int order, double x) {
  SplineCoef s = make_coef(order);
  double f = 0.0;
  if ((x > 0.0) && (x < (double)order)) {
    const int k = (int)x;
    for (int i = 0; i <= k; ++i) f = f + s.c[i] * ipow(x - (double)i, order - 1);
  }
  return f;
}

}  // namespace ermod

namespace ermod {
namespace {

// ---- solution mode's configuration check (check_mol_configuration) ------------------

struct CheckArgs {
  const double* sitepos;    // (3, numatm) as the frame gave them
  const double* agg_mass;   // [numatm] host-aggregate site masses, 0 elsewhere
  const double* site_mass;  // [numatm]
  const int* mbi0;
  int numatm, nummol;
  const int* tag;
  int nplace;
  int pos, str;  // insposition 2-5 or 0; insstructure 1 or 0
  double lw, up, lwstr, upstr;
  double inv3[3], len3;  // row 3 of the inverse cell, |cell axis 3|
  int ref_nh, ref_ns;
  const int* ref_atoms;    // [ref_nh]
  const double* ref_host;  // [ref_nh][4]
  const double* ref_slt;   // [ref_ns][4]
  DevStatus* status;
  int* skip;
};

// n sums over the block (fixed tree), returned to every thread
template <int N>
__device__ void block_sums(double (*red)[256], double (&v)[N]) {
  for (int c = 0; c < N; ++c) red[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int c = 0; c < N; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  for (int c = 0; c < N; ++c) v[c] = red[c][0];
  __syncthreads();
}

// rmsd_nofit (bestfit.F90:256-270) of a solute's sites (from atom a0) against points
// ref[s][0..2] with weights w(s)
template <class RefAt, class WAt>
__device__ double rmsd_nofit_dev(int n, RefAt ref, const double* __restrict__ pos, int a0, WAt w) {
  double W = 0.0, disp = 0.0;
  for (int s = 0; s < n; ++s) {
    W += w(s);
    double d2 = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double dx = pos[3 * (size_t)(a0 + s) + i] - ref(s, i);
      d2 += dx * dx;
    }
    disp += w(s) * d2;
  }
  return sqrt(disp / W);
}

// One CTA for the placements of a call.  The frame-wide parts first: the host
// aggregate's centre of mass (insposition 2-4; com_aggregate, insertion.F90:539-566), or
// the reference solute carried into the frame by the best fit of the reference host onto
// the frame's refspec atoms (insposition 5; engproc.F90:1099-1117).  Then a thread per
// placement applies the position test and, for a placement that passes, the structure
// test (insstructure 1: best-fit RMSD, engproc.F90:1127-1141); skip[p] = 1 where the
// reference sets out_of_range.  FP64 throughout; the block sums run in a fixed order.
__global__ void __launch_bounds__(256) config_check_kernel(CheckArgs A) {
  __shared__ double red[9][256];
  __shared__ double sfit[kMaxSoluteSites][3];  // the fitted reference solute (insposition 5)
  const double* X = A.sitepos;
  double ac[3] = {0.0, 0.0, 0.0};
  if (A.pos >= 2 && A.pos <= 4) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int a = threadIdx.x; a < A.numatm; a += blockDim.x) {
      const double w = A.agg_mass[a];
      if (w != 0.0) {
        v[0] += w;
        for (int c = 0; c < 3; ++c) v[c + 1] += w * X[3 * (size_t)a + c];
      }
    }
    block_sums<4>(red, v);
    for (int c = 0; c < 3; ++c) ac[c] = v[c + 1] / v[0];
  } else if (A.pos == 5) {
    // fit_a_rotate_b(refhost_natom, hostcrd, refhost_crd, refhost_weight, refslt_natom,
    // refslt_crd, refslt_bestfit): centres, then the centred sums of products
    double v[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < A.ref_nh; k += blockDim.x) {
      const double w = A.ref_host[4 * k + 3];
      const int at = A.ref_atoms[k];
      v[0] += w;
      for (int c = 0; c < 3; ++c) {
        v[1 + c] += w * X[3 * (size_t)at + c];
        v[4 + c] += w * A.ref_host[4 * k + c];
      }
    }
    block_sums<7>(red, v);
    double cf[3], cr[3];  // centres: frame host (the fit's reference), reference host
    for (int c = 0; c < 3; ++c) {
      cf[c] = v[1 + c] / v[0];
      cr[c] = v[4 + c] / v[0];
    }
    double S9[9];
    for (int c = 0; c < 9; ++c) S9[c] = 0.0;
    for (int k = threadIdx.x; k < A.ref_nh; k += blockDim.x) {
      const double w = A.ref_host[4 * k + 3];
      const int at = A.ref_atoms[k];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          S9[3 * j + i] += (X[3 * (size_t)at + i] - cf[i]) * (A.ref_host[4 * k + j] - cr[j]) * w;
    }
    block_sums<9>(red, S9);
    if (threadIdx.x == 0) {
      double S[3][3], q[4];
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) S[j][i] = S9[3 * j + i];
      bestfit::rotation_quaternion(S, q);
      for (int s = 0; s < A.ref_ns; ++s) {
        const double b[3] = {A.ref_slt[4 * s], A.ref_slt[4 * s + 1], A.ref_slt[4 * s + 2]};
        double o[3];
        bestfit::apply_fit(cf, cr, q, b, o);
        for (int c = 0; c < 3; ++c) sfit[s][c] = o[c];
      }
    }
    __syncthreads();
  }
  const int ns = A.ref_ns;
  const double* RS = A.ref_slt;
  auto wslt = [RS](int s) { return RS[4 * s + 3]; };
  for (int p = threadIdx.x; p < A.nplace; p += blockDim.x) {
    const int mol = A.tag[p] - 1;
    int out = 1;  // a tag out of range is never accumulated (the placement call reports it)
    if (mol >= 0 && mol < A.nummol) {
      const int a0 = A.mbi0[mol], n = A.mbi0[mol + 1] - a0;
      out = 0;
      if (A.pos >= 2 && A.pos <= 4) {  // relative_com (engproc.F90:1151-1172)
        double sm = 0.0, sc[3] = {0.0, 0.0, 0.0};
        for (int a = a0; a < a0 + n; ++a) {
          const double w = A.site_mass[a];
          sm += w;
          for (int c = 0; c < 3; ++c) sc[c] += w * X[3 * (size_t)a + c];
        }
        double dx[3];
        for (int c = 0; c < 3; ++c) dx[c] = sc[c] / sm - ac[c];
        double d;
        if (A.pos == 2) {
          d = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        } else {
          d = (A.inv3[0] * dx[0] + A.inv3[1] * dx[1] + A.inv3[2] * dx[2]) * A.len3;
          if (A.pos == 4) d = fabs(d);
        }
        out = (A.lw > d || d > A.up) ? 1 : 0;
      } else if (A.pos == 5 || A.str == 1) {
        if (n != ns) {  // numsite(tagslt) /= refslt_natom: 'eng_bug'
          atomicMin(&A.status->err_key, make_err_key(p, 0, ERMOD_E_ENG_BUG));
          out = 1;
        } else if (A.pos == 5) {
          const double d = rmsd_nofit_dev(ns, [](int s, int c) { return sfit[s][c]; }, X, a0, wslt);
          out = (A.lw > d || d > A.up) ? 1 : 0;
        }
      }
      if (!out && A.str == 1 && n == ns) {  // rmsd_bestfit(refslt_crd, the solute)
        double cref[3], cmol[3], q[4];
        bestfit::fit_transform(
            ns, [RS](int s, int c) { return RS[4 * s + c]; },
            [X, a0](int s, int c) { return X[3 * (size_t)(a0 + s) + c]; }, wslt, cref, cmol, q);
        double W = 0.0, disp = 0.0;
        for (int s = 0; s < ns; ++s) {
          const double b[3] = {X[3 * (size_t)(a0 + s)], X[3 * (size_t)(a0 + s) + 1], X[3 * (size_t)(a0 + s) + 2]};
          double o[3];
          bestfit::apply_fit(cref, cmol, q, b, o);
          double d2 = 0.0;
          for (int c = 0; c < 3; ++c) d2 += (o[c] - RS[4 * s + c]) * (o[c] - RS[4 * s + c]);
          W += wslt(s);
          disp += wslt(s) * d2;
        }
        const double d = sqrt(disp / W);
        out = (A.lwstr > d || d > A.upstr) ? 1 : 0;
      }
    }
    A.skip[p] = out;
  }
}

}  // namespace

cudaError_t launch_config_check(Engine& e, int nplace, const int* d_tag) {
  CheckArgs A{};
  A.sitepos = e.d_sitepos;
  A.agg_mass = e.d_agg_mass;
  A.site_mass = e.d_site_mass;
  A.mbi0 = e.d_mbi0;
  A.numatm = e.numatm;
  A.nummol = e.nummol;
  A.tag = d_tag;
  A.nplace = nplace;
  A.pos = e.cfg_pos;
  A.str = e.cfg_str;
  A.lw = e.cfg_lw;
  A.up = e.cfg_up;
  A.lwstr = e.cfg_lwstr;
  A.upstr = e.cfg_upstr;
  for (int c = 0; c < 3; ++c) A.inv3[c] = e.geom.invcl[2 + 3 * c];
  A.len3 = std::sqrt(e.cell[6] * e.cell[6] + e.cell[7] * e.cell[7] + e.cell[8] * e.cell[8]);
  A.ref_nh = e.ref_nh;
  A.ref_ns = e.ref_ns;
  A.ref_atoms = e.d_ref_atoms;
  A.ref_host = e.d_ref_host;
  A.ref_slt = e.d_ref_slt;
  A.status = e.d_status;
  A.skip = e.d_skip;
  config_check_kernel<<<1, 256, 0, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
