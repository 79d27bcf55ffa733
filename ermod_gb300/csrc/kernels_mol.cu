// kernels_mol.cu -- per-molecule solute-solvent energies, fused with the binning.
//
// One thread owns one solvent molecule (a "slot" of the frame's spatially sorted
// order) and G placements of the batch.  For each placement it computes
//   recip   sum over its sites of q * sum_{c1,c2,c3} theta theta theta phi(g - c)
//           (recpcal_energy, recpcal.F90:451-502), phi being the solute's PME potential;
//   real    LJ (4 switch forms) + q q erfc(beta r) / r against every solute site within
//           the cutoffs (get_pair_energy_block, realcal.F90:585-784), entered only when
//           the molecule is inside the solute's bounding sphere + cutoff, so the cell
//           list of the reference (realcal.F90:373-582) is not needed;
//   resid   -pi Q_u Q_j / (beta^2 V) (residual_ene, engproc.F90:859-869);
// then the FP64 total u = real + (resid + recip) (get_uv_energy, engproc.F90:736-753)
// is binned exactly as getiduv/binsearch do (engproc.F90:927-1020), with integer keys
// of the FP64 values, into a shared-memory histogram per placement (insdst,
// engproc.F90:813-830).  Per-species sum/min/max go to per-block partials reduced in
// a fixed tree, so every result is run-to-run deterministic.
//
// Mixed path: fixed-point positions, FP32 pair terms and grid gather, FP64 per-site and
// per-molecule totals.  FP64 path: everything in FP64 with the reference's formulas.
#include <cub/device/device_radix_sort.cuh>

#include "async_copy.cuh"
#include "engine.cuh"

namespace ermod {

struct LjK {  // switching constants (realcal.F90:629-642, 888-904)
  float lw2, up2, lw3, up3, lw6, up6, repA, repB, repC, attA, attB, attC, lw, up, ele2, den3;
};
// the same in FP64 (the FP64 path, and the mixed path's FP64 pair terms)
struct LjK64 {
  double lw2, up2, lw3, up3, lw6, up6, repA, repB, repC, attA, attB, attC, lw, up, ele2;
};

struct MolArgs {
  // frame, slot order
  const int4* site_pos;
  const float4* site_rec;
  const int* site_grid;
  const double* site_x;
  const double* site_w;
  const double* site_q;
  const int* slot_mol;
  const int* slot_site;
  const int* slot_species;
  const double* slot_qmol;
  const float* frame_scal;
  const int* mol_to_k;
  int slvmax, nummol;
  // LJ tables
  const double* ljene;
  const double* ljlensq;
  const float* ljene_f;
  const float* ljlensq_f;
  int T;
  int ldb;  // interleave stride of the mixed potential grids (placements per grid point)
  // energy coordinate
  const long long* uvkey;
  const int* uvkey_f;  // 32-bit keys of the edges rounded down to floats (FP32 totals)
  const int* spec;  // [numslv][3]
  int numslv, ermax, soln, mbin_mode;  // mbin_mode: 0 off, 1 error, 2 flag only
  int hist_global;  // finish kernel: histogram atomics straight into global memory (large ermax)
  // interaction parameters
  FrameGeom g;
  int ljswitch;
  double elecut, lwljcut, upljcut, screen;
  // FP32 constants of the mixed kernels, computed on the host
  float fxf[3];    // fixed-point unit per axis (box length / 2^32)
  float screen_f;  // Ewald beta
  float rc_f;      // max(elecut, upljcut)
  int bare;        // cltype 0: bare Coulomb within elecut (no cutoff when non-periodic), no reciprocal space
                   // or residual
  LjK k32;         // LJ switching constants
  LjK64 k64;
  double resid_fac;  // pi / screen^2 / volume
  // batch
  BatchArgs a;
  int ntile;
  DevStatus* status;
};

namespace {

template <typename T>
__device__ __forceinline__ T lj_low(int sw, const LjK& k, T eps, T sg2, T dist) {
  const T invr2 = sg2 / dist;
  const T invr6 = invr2 * invr2 * invr2;
  if (sw <= 1) return T(4) * eps * invr6 * (invr6 - T(1));
  const T s6 = sg2 * sg2 * sg2;
  if (sw == 2) {
    const T vdwa = invr6 * invr6 - s6 * s6 / (T(k.lw6) * T(k.up6));
    const T vdwb = invr6 - s6 / (T(k.lw3) * T(k.up3));
    return T(4) * eps * (vdwa - vdwb);
  }
  const T vdwa = invr6 * invr6 - s6 * s6 * T(k.repC);
  const T vdwb = invr6 - s6 * T(k.attC);
  return T(4) * eps * (vdwa - vdwb);
}

template <typename T>
__device__ __forceinline__ T lj_switch(int sw, const LjK& k, T eps, T sg2, T dist) {
  const T invr2 = sg2 / dist;
  const T invr6 = invr2 * invr2 * invr2;
  if (sw == 0) {
    const T dd = dist - T(k.up2), den = T(k.up2) - T(k.lw2);
    return T(4) * eps * invr6 * (invr6 - T(1)) * (T(2) * dist + T(k.up2) - T(3) * T(k.lw2)) * (dd * dd) /
           (den * den * den);
  }
  if (sw == 1) {
    const T swfac = (sqrt(dist) - T(k.lw)) / (T(k.up) - T(k.lw));
    const T s3 = swfac * swfac * swfac, s4 = s3 * swfac, s5 = s4 * swfac;
    return T(4) * eps * invr6 * (invr6 - T(1)) * (T(1) - T(10) * s3 + T(15) * s4 - T(6) * s5);
  }
  const T s6 = sg2 * sg2 * sg2;
  if (sw == 2) {
    const T invr3 = sqrt(invr6), s3 = sqrt(s6);
    const T a = invr6 - s6 / T(k.up6), b = invr3 - s3 / T(k.up3);
    const T vdwa = T(k.up6) / (T(k.up6) - T(k.lw6)) * (a * a);
    const T vdwb = T(k.up3) / (T(k.up3) - T(k.lw3)) * (b * b);
    return T(4) * eps * (vdwa - vdwb);
  }
  const T swfac = sqrt(dist) - T(k.lw);
  const T f3 = swfac * swfac * swfac, f4 = f3 * swfac;
  const T vdwa = invr6 * invr6 - s6 * s6 * (T(k.repA) * f3 + T(k.repB) * f4 + T(k.repC));
  const T vdwb = invr6 - s6 * (T(k.attA) * f3 + T(k.attB) * f4 + T(k.attC));
  return T(4) * eps * (vdwa - vdwb);
}

__device__ __forceinline__ double lj_low64(int sw, const LjK64& k, double eps, double sg2, double dist) {
  const double invr2 = sg2 / dist;
  const double invr6 = invr2 * invr2 * invr2;
  if (sw <= 1) return 4.0 * eps * invr6 * (invr6 - 1.0);
  const double s6 = sg2 * sg2 * sg2;
  if (sw == 2) {
    const double vdwa = invr6 * invr6 - s6 * s6 / (k.lw6 * k.up6);
    const double vdwb = invr6 - s6 / (k.lw3 * k.up3);
    return 4.0 * eps * (vdwa - vdwb);
  }
  const double vdwa = invr6 * invr6 - s6 * s6 * k.repC;
  const double vdwb = invr6 - s6 * k.attC;
  return 4.0 * eps * (vdwa - vdwb);
}

__device__ __forceinline__ double lj_switch64(int sw, const LjK64& k, double eps, double sg2, double dist) {
  const double invr2 = sg2 / dist;
  const double invr6 = invr2 * invr2 * invr2;
  if (sw == 0) {
    const double dd = dist - k.up2, den = k.up2 - k.lw2;
    return 4.0 * eps * invr6 * (invr6 - 1.0) * (2.0 * dist + k.up2 - 3.0 * k.lw2) * (dd * dd) / (den * den * den);
  }
  if (sw == 1) {
    const double swfac = (sqrt(dist) - k.lw) / (k.up - k.lw);
    const double s3 = swfac * swfac * swfac, s4 = s3 * swfac, s5 = s4 * swfac;
    return 4.0 * eps * invr6 * (invr6 - 1.0) * (1.0 - 10.0 * s3 + 15.0 * s4 - 6.0 * s5);
  }
  const double s6 = sg2 * sg2 * sg2;
  if (sw == 2) {
    const double invr3 = sqrt(invr6), s3 = sqrt(s6);
    const double a = invr6 - s6 / k.up6, b = invr3 - s3 / k.up3;
    const double vdwa = k.up6 / (k.up6 - k.lw6) * (a * a);
    const double vdwb = k.up3 / (k.up3 - k.lw3) * (b * b);
    return 4.0 * eps * (vdwa - vdwb);
  }
  const double swfac = sqrt(dist) - k.lw;
  const double f3 = swfac * swfac * swfac, f4 = f3 * swfac;
  const double vdwa = invr6 * invr6 - s6 * s6 * (k.repA * f3 + k.repB * f4 + k.repC);
  const double vdwb = invr6 - s6 * (k.attA * f3 + k.attB * f4 + k.attC);
  return 4.0 * eps * (vdwa - vdwb);
}

__host__ __device__ __forceinline__ void gmx_params(int pw, double lw, double up, double& A, double& B, double& C) {
  const double df = up - lw;
  double upp2 = 1.0, upp = 1.0;
  for (int i = 0; i < pw + 2; ++i) upp2 *= up;
  for (int i = 0; i < pw; ++i) upp *= up;
  A = -(double)pw * ((double)(pw + 4) * up - (double)(pw + 1) * lw) / (upp2 * (df * df)) / 3.0;
  B = (double)pw * ((double)(pw + 3) * up - (double)(pw + 1) * lw) / (upp2 * (df * df * df)) / 4.0;
  C = 1.0 / upp - A * (df * df * df) - B * (df * df * df * df);
}

__host__ __device__ __forceinline__ LjK64 make_k64(const MolArgs& A) {
  LjK64 k;
  k.lw = A.lwljcut;
  k.up = A.upljcut;
  k.lw2 = A.lwljcut * A.lwljcut;
  k.up2 = A.upljcut * A.upljcut;
  k.lw3 = A.lwljcut * A.lwljcut * A.lwljcut;
  k.up3 = A.upljcut * A.upljcut * A.upljcut;
  k.lw6 = k.lw3 * k.lw3;
  k.up6 = k.up3 * k.up3;
  gmx_params(12, A.lwljcut, A.upljcut, k.repA, k.repB, k.repC);
  gmx_params(6, A.lwljcut, A.upljcut, k.attA, k.attB, k.attC);
  k.ele2 = A.elecut * A.elecut;
  return k;
}

__host__ __device__ __forceinline__ LjK to_f32(const LjK64& d) {
  LjK k;
  k.lw2 = (float)d.lw2; k.up2 = (float)d.up2; k.lw3 = (float)d.lw3; k.up3 = (float)d.up3;
  k.lw6 = (float)d.lw6; k.up6 = (float)d.up6; k.repA = (float)d.repA; k.repB = (float)d.repB;
  k.repC = (float)d.repC; k.attA = (float)d.attA; k.attB = (float)d.attB; k.attC = (float)d.attC;
  k.lw = (float)d.lw; k.up = (float)d.up; k.ele2 = (float)d.ele2; k.den3 = 0.f;
  return k;
}

__device__ __forceinline__ int wrapi(int x, int K) {
  if (x < 0) x += K;
  if (x >= K) x -= K;
  return x;
}

// fixed-tree block reductions over blockDim.x (power of two) entries
__device__ __forceinline__ double block_sum(double* sm, double v) {
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sm[threadIdx.x] += sm[threadIdx.x + st];
    __syncthreads();
  }
  const double r = sm[0];
  __syncthreads();
  return r;
}
__device__ __forceinline__ long long block_min(long long* sm, long long v) {
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sm[threadIdx.x] = min(sm[threadIdx.x], sm[threadIdx.x + st]);
    __syncthreads();
  }
  const long long r = sm[0];
  __syncthreads();
  return r;
}
__device__ __forceinline__ long long block_max(long long* sm, long long v) {
  sm[threadIdx.x] = v;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sm[threadIdx.x] = max(sm[threadIdx.x], sm[threadIdx.x + st]);
    __syncthreads();
  }
  const long long r = sm[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double key_to_double(long long k) {
  k = k ^ ((k >> 63) & 0x7fffffffffffffffll);
  return __longlong_as_double(k);
}


// getiduv / binsearch for one molecule: returns the status code (0 = binned) and ret,
// the count of edges strictly below u (bin = sp_off + ret - 1).
__device__ __forceinline__ int bin_molecule(const MolArgs& A, double u, int species, int sp_off, int sp_n,
                                            int sp_soft, int& ret) {
  ret = 0;
  if (species < 1 || species > A.numslv) return ERMOD_E_ENG_CNS;
  if (u != u) return ERMOD_E_ENG_MIN;
  const long long ku = ordered_key(u);
  const long long* keys = A.uvkey + sp_off;
  int lo = 0, hi = sp_n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(keys + mid) < ku)
      lo = mid + 1;
    else
      hi = mid;
  }
  ret = lo;
  if (ret <= 0) return ERMOD_E_ENG_MIN;
  if (A.soln && ret > sp_soft) return ERMOD_E_ENG_SFT;
  if (ret == sp_n && u < 1.0e3 && A.mbin_mode != 0) {
    if (A.mbin_mode == 1) return ERMOD_W_MBIN;
    atomicOr(&A.status->mbin_hit, 1);
  }
  return 0;
}

// warp-aggregated shared-memory histogram increment
__device__ __forceinline__ void hist_add(int* h, int bin) {
  const unsigned am = __activemask();
  const unsigned peers = __match_any_sync(am, bin);
  const int leader = __ffs(peers) - 1;
  if ((threadIdx.x & 31) == leader) atomicAdd(&h[bin], __popc(peers));
}

// FP32 pair terms larger than these (kcal/mol) are recomputed in FP64.  Below them an
// FP32 term is within a few units in the last place (the LJ term's sigma^12 amplifies the
// distance's rounding 6-fold; erfcf is within 4 ulp), 5e-6 kcal/mol at most; above them the
// FP32 rounding, and the fixed-point quantisation of the displacement (2.3e-8 A at
// L = 99.5 A), would grow with the term up to the 1e10 kcal/mol of overlapping pairs.
constexpr float kFp64Lj = 8.0f;
constexpr float kFp64Coulomb = 16.0f;
constexpr int kPairLj = 1, kPairCoulomb = 2;  // the parts of a pair evaluated in FP64

// parts of one solute-solvent site pair in FP64, as the FP64 path computes them: minimum
// image of the FP64 wrapped coordinates (realcal.F90:202-209), LJ with the switch form
// (realcal.F90:686-770) and the screened or bare Coulomb term (realcal.F90:771-782, 245)
__device__ __forceinline__ double pair_fp64(const MolArgs& A, int idx, const double* __restrict__ ux, double qu,
                                         int tu, int parts) {
  double dist = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double h = 0.5 * A.g.L[i];
    const double x = fabs(A.site_x[3 * (size_t)idx + i] - ux[i]);
    const double d = A.g.periodic ? h - fabs(h - x) : x;
    dist += d * d;
  }
  const int tv = A.site_pos[idx].w;
  double e = 0.0;
  const double ljeps = A.ljene[tv + A.T * tu];
  if ((parts & kPairLj) && ljeps > 0) {
    const double sg2 = A.ljlensq[tv + A.T * tu];
    if (dist <= A.k64.lw2)
      e += lj_low64(A.ljswitch, A.k64, ljeps, sg2, dist);
    else if (dist <= A.k64.up2)
      e += lj_switch64(A.ljswitch, A.k64, ljeps, sg2, dist);
  }
  if (parts & kPairCoulomb) {
    if (A.bare) {
      if (dist < A.k64.ele2) e += qu * A.site_q[idx] / sqrt(dist);
    } else if (dist <= A.k64.ele2) {
      const double r = sqrt(dist);
      e += qu * A.site_q[idx] * (1.0 - erf(A.screen * r)) / r;
    }
  }
  return e;
}

// FP64 pairs recorded per thread by the finish kernel's first pass (see mol_finish_kernel)
constexpr int kBigPerThread = 8;
// that pass's scratch (ints): the recorded pairs, their compacted list (16-bit), the
// threads' first sites and one double per thread
constexpr int kFinishScratchInts = 256 * kBigPerThread + 256 * kBigPerThread / 2 + 256 + 2 * 256;
// the dynamic shared memory of the finish kernel before its edge keys: the block
// histograms (when in shared memory) or the FP64 pass's scratch, whichever is larger
__host__ __device__ __forceinline__ int finish_region_ints(int G, int ermax, int hist_global) {
  const int h = hist_global ? 0 : G * ermax;
  return h > kFinishScratchInts ? h : kFinishScratchInts;
}
// a recorded pair: its FP64 parts (2 bits), placement j of the block (3 bits), solute site
// (8 bits), site of the solvent molecule (13 bits)
__device__ __forceinline__ int big_item(int parts, int j, int su, int s) {
  return (parts << 24) | (j << 21) | (su << 13) | s;
}

// real-space LJ + screened Coulomb of one molecule against solute b (mixed path):
// fixed-point displacements and FP32 pair terms, summed as a float-float number.  An FP32
// LJ or Coulomb term above kFp64Lj / kFp64Coulomb in magnitude (or not finite) is left out
// of the sum and counted in nbig (in the thread's scan order); the count's values in
// [win, win + kBigPerThread) are recorded with their parts in items[count - win], and bit j
// of fix is set.  kSum: sum the FP32 terms (the first pass); else only record (the later
// rounds of a thread with more pairs than one round takes).
constexpr int kMolSiteCache = 3;  // molecule sites held in registers by the real-space pass

template <bool kSum>
__device__ __forceinline__ ff real_mixed(const MolArgs& A, const BatchArgs& a, int b, int s0, int ns,
                                         const LjK& k32, float rcut, int4 p0, int4 u0, int j, int* items,
                                         int win, int& nbig, unsigned& fix) {
  const size_t ub = (size_t)b * kMaxSoluteSites;
  const float fx = A.fxf[0], fy = A.fxf[1], fz = A.fxf[2];
  const float dx = (float)(int)((unsigned)p0.x - (unsigned)u0.x) * fx;
  const float dy = (float)(int)((unsigned)p0.y - (unsigned)u0.y) * fy;
  const float dz = (float)(int)((unsigned)p0.z - (unsigned)u0.z) * fz;
  ff real{0.f, 0.f};
  if (dx * dx + dy * dy + dz * dz > rcut * rcut) return real;
  const int nu = a.u_nsite[b];
  const float beta = A.screen_f;
  // one pair (solute site su at up with charge qu, molecule site s at vp with charge qv)
  auto pair = [&](int su, const int4& up, float qu, int s, const int4& vp, float qv) {
    const float ex = (float)(int)((unsigned)vp.x - (unsigned)up.x) * fx;
    const float ey = (float)(int)((unsigned)vp.y - (unsigned)up.y) * fy;
    const float ez = (float)(int)((unsigned)vp.z - (unsigned)up.z) * fz;
    const float r2 = ex * ex + ey * ey + ez * ez;
    float elj = 0.f, eco = 0.f;
    const float ljeps = A.ljene_f[vp.w + A.T * up.w];
    if (ljeps > 0.f) {
      const float sg2 = A.ljlensq_f[vp.w + A.T * up.w];
      if (r2 <= k32.lw2)
        elj = lj_low<float>(A.ljswitch, k32, ljeps, sg2, r2);
      else if (r2 <= k32.up2)
        elj = lj_switch<float>(A.ljswitch, k32, ljeps, sg2, r2);
    }
    if (A.bare) {
      if (r2 < k32.ele2) eco = qu * qv / sqrtf(r2);  // realcal_bare
    } else if (r2 <= k32.ele2) {
      const float r = sqrtf(r2);
      eco = qu * qv * erfcf(beta * r) / r;
    }
    // parts too large for FP32 (the comparisons are false for NaN and inf)
    const int parts = (fabsf(elj) <= kFp64Lj ? 0 : kPairLj) | (fabsf(eco) <= kFp64Coulomb ? 0 : kPairCoulomb);
    if (kSum) {
      if (!(parts & kPairLj)) real = ff_add(real, elj);
      if (!(parts & kPairCoulomb)) real = ff_add(real, eco);
    }
    if (parts) {
      const int r = nbig - win;
      if (r >= 0 && r < kBigPerThread) items[r] = big_item(parts, j, su, s);
      ++nbig;
      fix |= 1u << j;
    }
  };
  if (ns <= kMolSiteCache) {
    // small molecules (water): their sites' positions and charges held in registers for
    // every solute site
    int4 vpc[kMolSiteCache];
    float qvc[kMolSiteCache];
#pragma unroll
    for (int s = 0; s < kMolSiteCache; ++s)
      if (s < ns) {
        vpc[s] = A.site_pos[s0 + s];
        qvc[s] = A.site_rec[s0 + s].w;
      }
    for (int su = 0; su < nu; ++su) {
      const int4 up = a.u_pos[ub + su];
      const float qu = a.u_qf[ub + su];
#pragma unroll
      for (int s = 0; s < kMolSiteCache; ++s)
        if (s < ns) pair(su, up, qu, s, vpc[s], qvc[s]);
    }
  } else {
    for (int su = 0; su < nu; ++su) {
      const int4 up = a.u_pos[ub + su];
      const float qu = a.u_qf[ub + su];
      for (int s = 0; s < ns; ++s) pair(su, up, qu, s, A.site_pos[s0 + s], A.site_rec[s0 + s].w);
    }
  }
  return real;
}

constexpr long long kKeyPosInf = 0x7ff0000000000000ll;
constexpr long long kKeyNegInf = (long long)0x800fffffffffffffull;  // ordered key of -inf

// the plain FP64 path: one placement group per block row, one solvent molecule per thread
template <int P>
__global__ void __launch_bounds__(256) mol_energy_kernel(MolArgs A) {
  extern __shared__ int smem_hist[];  // [G][ermax]
  __shared__ double sred[256];
  __shared__ long long skey[256];
  const int tile = blockIdx.x;
  const int bgrp = blockIdx.y;
  const BatchArgs& a = A.a;
  const int G = a.G;
  const int m = tile * blockDim.x + threadIdx.x;
  const bool valid = m < A.slvmax;
  for (int i = threadIdx.x; i < G * A.ermax; i += blockDim.x) smem_hist[i] = 0;
  __syncthreads();

  int k = -1, s0 = 0, ns = 0, species = 0;
  double qmol = 0.0;
  if (valid) {
    k = A.slot_mol[m];
    s0 = A.slot_site[m];
    ns = A.slot_site[m + 1] - s0;
    species = A.slot_species[m];
    qmol = A.slot_qmol[m];
  }
  const FrameGeom& g = A.g;
  const int K1 = g.K[0], K2 = g.K[1], K3 = g.K[2];
  const size_t gridn = (size_t)K1 * K2 * K3;
  const LjK64 k64 = make_k64(A);
  const double rc = fmax(A.elecut, A.upljcut);
  const float mol_r = A.frame_scal[0];
  int sp_off = 0, sp_n = 1, sp_soft = 1;
  if (valid && species >= 1 && species <= A.numslv) {
    sp_off = A.spec[3 * (species - 1)];
    sp_n = A.spec[3 * (species - 1) + 1];
    sp_soft = A.spec[3 * (species - 1) + 2];
  }

  for (int gi = 0; gi < G; ++gi) {
    const int b = bgrp * G + gi;
    if (b >= a.nb) break;  // uniform across the block
    const int tg = a.tagslt[b] - 1;
    const int kskip = (tg >= 0 && tg < A.nummol) ? A.mol_to_k[tg] : -2;
    // a placement rejected by check_mol_configuration has no molecule (engproc.F90:690-691)
    const bool active = valid && (k != kskip) && !(a.skip && a.skip[b]);
    double u = 0.0;
    if (active) {
      // ---- reciprocal part ----
      double recip = 0.0;
      if (!A.bare) {  // bare Coulomb: no reciprocal part
        const double* phi = a.phi64 + (size_t)b * gridn;
        for (int s = 0; s < ns; ++s) {
          const int idx = s0 + s;
          const double chr = A.site_q[idx];
          const double* w = A.site_w + (size_t)idx * 3 * P;
          const int gp = A.site_grid[idx];
          const int g1 = gp & 1023, g2 = (gp >> 10) & 1023, g3 = (gp >> 20) & 1023;
          for (int c3 = 0; c3 < P; ++c3) {
            const double fac1 = chr * w[2 * P + c3];
            const int z = wrapi(g3 - c3, K3);
            for (int c2 = 0; c2 < P; ++c2) {
              const double fac2 = fac1 * w[P + c2];
              const int y = wrapi(g2 - c2, K2);
              const double* row = phi + ((size_t)z * K2 + y) * K1;
              for (int c1 = 0; c1 < P; ++c1) {
                const double fac3 = fac2 * w[c1];
                recip = recip + fac3 * row[wrapi(g1 - c1, K1)];
              }
            }
          }
        }
      }
      // ---- real space ----
      double real = 0.0;
      const int nu = a.u_nsite[b];
      const size_t ub = (size_t)b * kMaxSoluteSites;
      const float rcut = (float)rc + a.u_radius[b] + mol_r;
      double d0 = 0.0;
      for (int i = 0; i < 3; ++i) {
        const double h = 0.5 * g.L[i];
        const double x = fabs(A.site_x[3 * (size_t)s0 + i] - a.u_x[ub * 3 + i]);
        const double d = g.periodic ? h - fabs(h - x) : x;
        d0 += d * d;
      }
      if (d0 <= (double)rcut * (double)rcut) {
        for (int su = 0; su < nu; ++su) {
          const double* ux = a.u_x + (ub + su) * 3;
          const double qu = a.u_q[ub + su];
          const int tu = a.u_pos[ub + su].w;
          for (int s = 0; s < ns; ++s) {
            const int idx = s0 + s;
            double dist = 0.0;
            for (int i = 0; i < 3; ++i) {  // minimum image only when periodic (realcal.F90:202-209)
              const double h = 0.5 * g.L[i];
              const double x = fabs(A.site_x[3 * (size_t)idx + i] - ux[i]);
              const double d = g.periodic ? h - fabs(h - x) : x;
              dist += d * d;
            }
            const int tv = A.site_pos[idx].w;
            const double ljeps = A.ljene[tv + A.T * tu];
            if (ljeps > 0) {
              const double sg2 = A.ljlensq[tv + A.T * tu];
              if (dist <= k64.lw2)
                real += lj_low64(A.ljswitch, k64, ljeps, sg2, dist);
              else if (dist <= k64.up2)
                real += lj_switch64(A.ljswitch, k64, ljeps, sg2, dist);
            }
            if (A.bare) {
              if (dist < k64.ele2) real += qu * A.site_q[idx] / sqrt(dist);  // realcal_bare
            } else if (dist <= k64.ele2) {
              const double r = sqrt(dist);
              real += qu * A.site_q[idx] * (1.0 - erf(A.screen * r)) / r;
            }
          }
        }
      }
      // residual_ene + assembly (engproc.F90:741-752)
      double epcl;
      if (A.bare)
        epcl = 0.0;  // residual_ene returns without a term for bare Coulomb
      else
        epcl = kPi * a.u_qmol[b] * qmol / A.screen / A.screen / g.volume;
      double pairep = -epcl;
      pairep = pairep + recip;
      u = real + pairep;
      // ---- getiduv / binsearch ----
      int ret = 0;
      const int code = bin_molecule(A, u, species, sp_off, sp_n, sp_soft, ret);
      if (code)
        atomicMin(&A.status->err_key, make_err_key(a.b0 + b, k + 1, code));
      else
        hist_add(smem_hist + gi * A.ermax, sp_off + ret - 1);
      if (a.uvengy_out) a.uvengy_out[(size_t)(a.b0 + b) * (A.slvmax + 1) + k + 1] = u;
    } else if (valid && a.uvengy_out) {
      a.uvengy_out[(size_t)(a.b0 + b) * (A.slvmax + 1) + k + 1] = 0.0;
    }
    // per-species partials {sum, min, max} of this block (fixed-tree reductions)
    for (int sp = 1; sp <= A.numslv; ++sp) {
      const bool mine = active && species == sp;
      const double s = block_sum(sred, mine ? u : 0.0);
      const long long mn = block_min(skey, mine ? ordered_key(u) : kKeyPosInf);
      const long long mx = block_max(skey, mine ? ordered_key(u) : kKeyNegInf);
      if (threadIdx.x == 0) {
        double* pt = a.part + (((size_t)b * A.ntile + tile) * A.numslv + (sp - 1)) * 3;
        pt[0] = s;
        pt[1] = key_to_double(mn);
        pt[2] = key_to_double(mx);
      }
    }
  }
  __syncthreads();
  // flush the block's histograms
  for (int gi = 0; gi < G; ++gi) {
    const int b = bgrp * G + gi;
    if (b >= a.nb) break;
    const int* h = smem_hist + gi * A.ermax;
    int* out = a.hist + (size_t)b * A.ermax;
    for (int i = threadIdx.x; i < A.ermax; i += blockDim.x) {
      const int c = h[i];
      if (c) atomicAdd(out + i, c);
    }
  }
}


// ---- TMA + mbarrier helpers (inline PTX, sm_90+ forms, valid on sm_103a) -------------

// Mixed path, step 1 -- gather by bricks.  CTA per (kBrickX x kBrickY x kBrickZ brick of the
// PME grid, run of placement groups of 4).  One 5-D TMA box copy per group brings the
// brick's stencil halo of the group's interleaved potential grids into shared memory as
// [z][y][x][4], in kGatherStages buffers so that the next groups' copies are in flight
// while this one is used; each thread takes a site of the brick (its B-spline weights
// computed once for all groups, FP32 stable recursion) and accumulates
// q theta theta theta phi for the four placements with one 16-byte shared load per
// stencil point.
constexpr int kGatherThreads = 256;
constexpr int kGatherStages = 2;  // halo buffers (TMA copies in flight) per gather CTA

template <int P>
__device__ __forceinline__ void site_setup(int site, const float4* __restrict__ site_rec,
                                           const int* __restrict__ site_grid, int K1, int K2, int K3, int ox,
                                           int oy, int oz, int BX, float (&w1)[P], float (&w2)[P],
                                           float (&w3)[P], int& base, float& q) {
  constexpr int BY = kBrickY + P - 1;
  const float4 rec = site_rec[site];
  const int gp = site_grid[site];
  bspline_w<P>(rec.x, w1);
  bspline_w<P>(rec.y, w2);
  bspline_w<P>(rec.z, w3);
  int g1 = gp & 1023, g2 = (gp >> 10) & 1023, g3 = (gp >> 20) & 1023;
  if (g1 >= K1) g1 -= K1;
  if (g2 >= K2) g2 -= K2;
  if (g3 >= K3) g3 -= K3;
  base = ((g3 - oz) * BY + (g2 - oy)) * BX + (g1 - ox);  // stencil c covers l0 - c
  q = rec.w;
}

template <int P>
__device__ __forceinline__ float4 site_stencil(const float4* __restrict__ halo, int base, int BX,
                                               const float (&w1)[P], const float (&w2)[P], const float (&w3)[P]) {
  constexpr int BY = kBrickY + P - 1;
  constexpr int U3 = P <= 4 ? P : 1;  // higher orders: keep the register footprint bounded
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll U3
  for (int c3 = 0; c3 < P; ++c3) {
#pragma unroll
    for (int c2 = 0; c2 < P; ++c2) {
      const float w32 = w3[c3] * w2[c2];
      const float4* row = halo + base - (c3 * BY + c2) * BX;
#pragma unroll
      for (int c1 = 0; c1 < P; ++c1) {
        const float w = w32 * w1[c1];
        const float4 v = row[-c1];
        acc.x = fmaf(w, v.x, acc.x);
        acc.y = fmaf(w, v.y, acc.y);
        acc.z = fmaf(w, v.z, acc.z);
        acc.w = fmaf(w, v.w, acc.w);
      }
    }
  }
  return acc;
}

template <int P>
__global__ void __launch_bounds__(kGatherThreads) gather_tma_kernel(
    const __grid_constant__ CUtensorMap tmap, int nb, int groups_per_cta, const float4* __restrict__ site_rec,
    const int* __restrict__ site_grid, const int* __restrict__ brick_site, const int* __restrict__ brick_start,
    int K1, int K2, int K3, int nbx, int nby, int BX, int ldb, float* __restrict__ site_e, DevStatus* status) {
  constexpr int BY = kBrickY + P - 1, BZ = kBrickZ + P - 1;
  extern __shared__ unsigned char smem_raw[];
  __shared__ unsigned long long bar[kGatherStages];
  const int npt = BZ * BY * BX;
  // kGatherStages halo buffers [z][y][x] of float4 (the four placements of a group),
  // 128-byte aligned; group g lands in buffer (g - g_begin) % kGatherStages
  float4* halo_base = reinterpret_cast<float4*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  const int hstride = (npt + 7) & ~7;  // float4 elements, a multiple of 128 bytes
  const int brick = blockIdx.x;
  const int bx = brick % nbx, by = (brick / nbx) % nby, bz = brick / (nbx * nby);
  const int g_begin = blockIdx.y * groups_per_cta;
  const int g_end = min((nb + 3) / 4, g_begin + groups_per_cta);
  const uint32_t box_bytes = (uint32_t)(npt * sizeof(float4));
  if (threadIdx.x == 0) {
    for (int i = 0; i < kGatherStages; ++i) mbar_init(&bar[i], 1);
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();
  // padded coordinates: the halo of brick (bx, by, bz) starts at (kBrickX bx,
  // kBrickY by, kBrickZ bz); the innermost box coordinate (the placement within the
  // group) is 0
  if (threadIdx.x == 0) {
    for (int g = g_begin; g < min(g_end, g_begin + kGatherStages); ++g) {
      const int st = g - g_begin;
      mbar_expect_tx(&bar[st], box_bytes);
      tma_load_5d(halo_base + (size_t)st * hstride, &tmap, 0, bx * kBrickX, by * kBrickY, bz * kBrickZ, g, &bar[st]);
    }
  }
  const int h = P - 1;
  const int ox = bx * kBrickX - h, oy = by * kBrickY - h, oz = bz * kBrickZ - h;
  const int s_begin = brick_start[brick], s_end = brick_start[brick + 1];
  const int n = s_end - s_begin;
  // Site-to-thread map.  A 16-byte shared load is served 8 lanes at a time, and the
  // 8 lanes are conflict free when their halo indices differ mod 8; every stencil
  // point shifts all lanes' indices by the same offset.  So the brick's sites are
  // bucketed by (stencil base index mod 8), and lane t takes entry t / 8 of bucket t % 8.
  // Bricks with more sites than threads keep the plain order.
  __shared__ int sbucket[8][kGatherThreads / 8];
  __shared__ int scnt[8];
  __shared__ int sovf[kGatherThreads];
  __shared__ int novf;
  const bool bucketed = n <= (int)blockDim.x;
  int site0 = -1;
  if (bucketed) {
    if (threadIdx.x < 8) scnt[threadIdx.x] = 0;
    if (threadIdx.x == 0) novf = 0;
    __syncthreads();
    if ((int)threadIdx.x < n) {
      const int site = brick_site[s_begin + threadIdx.x];
      const int gp = site_grid[site];
      int g1 = gp & 1023, g2 = (gp >> 10) & 1023, g3 = (gp >> 20) & 1023;
      if (g1 >= K1) g1 -= K1;
      if (g2 >= K2) g2 -= K2;
      if (g3 >= K3) g3 -= K3;
      const int r = ((((g3 - oz) * BY + (g2 - oy)) * BX + (g1 - ox)) & 7);
      const int pos = atomicAdd(&scnt[r], 1);
      if (pos < (int)(kGatherThreads / 8))
        sbucket[r][pos] = site;
      else
        sovf[atomicAdd(&novf, 1)] = site;
    }
    __syncthreads();
    const int r = threadIdx.x & 7, k = threadIdx.x >> 3;
    if (k < scnt[r] && k < (int)(kGatherThreads / 8)) site0 = sbucket[r][k];
  } else if ((int)threadIdx.x < n) {
    site0 = brick_site[s_begin + threadIdx.x];
  }
  // this thread's site, set up once for every group
  float w1[P], w2[P], w3[P];
  int base = 0;
  float q = 0.f;
  if (site0 >= 0) site_setup<P>(site0, site_rec, site_grid, K1, K2, K3, ox, oy, oz, BX, w1, w2, w3, base, q);
  const int n_extra = bucketed ? novf : max(0, n - (int)blockDim.x);
  for (int g = g_begin; g < g_end; ++g) {
    const int slot = (g - g_begin) % kGatherStages;
    const uint32_t parity = (uint32_t)(((g - g_begin) / kGatherStages) & 1);
    bool ok = false;
    for (long it = 0; it < kWaitLimit; ++it)
      if (mbar_try_wait(&bar[slot], parity)) {
        ok = true;
        break;
      }
    if (!__syncthreads_and(ok)) {  // flag, let the other copies in flight land (bounded), leave
      if (threadIdx.x == 0) atomicOr(&status->range_fault, 2);
      for (int g2 = g + 1; g2 < min(g_end, g + kGatherStages); ++g2) {
        const int s2 = (g2 - g_begin) % kGatherStages;
        const uint32_t p2 = (uint32_t)(((g2 - g_begin) / kGatherStages) & 1);
        for (long it = 0; it < kWaitLimit; ++it)
          if (mbar_try_wait(&bar[s2], p2)) break;
      }
      return;
    }
    const float4* halo = halo_base + (size_t)slot * hstride;
    const int b0 = 4 * g;
    if (site0 >= 0) {
      const float4 acc = site_stencil<P>(halo, base, BX, w1, w2, w3);
      *reinterpret_cast<float4*>(site_e + (size_t)site0 * ldb + b0) =
          make_float4(q * acc.x, q * acc.y, q * acc.z, q * acc.w);
    }
    for (int i = threadIdx.x; i < n_extra; i += blockDim.x) {  // bucket overflow / crowded bricks
      const int site = bucketed ? sovf[i] : brick_site[s_begin + blockDim.x + i];
      float v1[P], v2[P], v3[P];
      int bs;
      float qs;
      site_setup<P>(site, site_rec, site_grid, K1, K2, K3, ox, oy, oz, BX, v1, v2, v3, bs, qs);
      const float4 acc = site_stencil<P>(halo, bs, BX, v1, v2, v3);
      *reinterpret_cast<float4*>(site_e + (size_t)site * ldb + b0) =
          make_float4(qs * acc.x, qs * acc.y, qs * acc.z, qs * acc.w);
    }
    __syncthreads();  // halo[slot] consumed: the copy of group g + kGatherStages may land in it
    if (threadIdx.x == 0 && g + kGatherStages < g_end) {
      fence_proxy_async_smem();
      mbar_expect_tx(&bar[slot], box_bytes);
      tma_load_5d(halo_base + (size_t)slot * hstride, &tmap, 0, bx * kBrickX, by * kBrickY, bz * kBrickZ, g + kGatherStages,
                  &bar[slot]);
    }
  }
}


// The number of a species' edges e below u = hi + lo, given pos, the number of edges
// whose float keys rd(e) lie below key32(hi) (kk: the species' float keys, uvkey: its
// FP64 edges as ordered keys).  The two counts can differ only for an edge within one
// float step of hi; such an edge is compared exactly in FP64 (e - hi is exact there, and
// lo is a float), so the bin is the one the FP64 value hi + lo takes against the FP64
// edges (getiduv/binsearch, engproc.F90:927-1020).
// (The FP64 comparisons sit in a function of their own, called only for a total that near
// an edge: inline, the compiler would issue them predicated for every molecule, and an
// FP64 instruction costs GB300 about 64 times an FP32 one even when no lane executes it.)
__device__ __noinline__ int exact_count_near(const long long* __restrict__ uvkey, const int* kk, int n, int pos,
                                            int khi, float hi, float lo) {
  while (pos > 0 && kk[pos - 1] >= khi - 2) {  // counted, but maybe not below u
    if (key_to_double(__ldg(uvkey + pos - 1)) - (double)hi < (double)lo) break;
    --pos;
  }
  while (pos < n && kk[pos] <= khi + 2) {  // not counted, but maybe below u
    if (!(key_to_double(__ldg(uvkey + pos)) - (double)hi < (double)lo)) break;
    ++pos;
  }
  return pos;
}
__device__ __forceinline__ int exact_count(const long long* __restrict__ uvkey, const int* kk, int n, int pos,
                                           int khi, float hi, float lo) {
  const bool near = (pos > 0 && kk[pos - 1] >= khi - 2) || (pos < n && kk[pos] <= khi + 2);
  return near ? exact_count_near(uvkey, kk, n, pos, khi, hi, lo) : pos;
}

// the finish kernel's per-species partials of its block (see mol_finish_kernel)
template <int G, bool kSum>
__device__ __forceinline__ void species_partials(const MolArgs& A, const BatchArgs& a, const float (*su)[256],
                                                 const float (*sul)[256], const unsigned char* sspec, int g0, int ng,
                                                 int tile) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int pr = warp; pr < ng * A.numslv; pr += blockDim.x / 32) {
    const int j = pr / A.numslv, sp = pr % A.numslv + 1;
    long long mn = kFfKeyNone, mx = kFfKeyNoneMax;
    double s = 0.0;
    for (int t = lane; t < blockDim.x; t += 32) {
      const float v = su[j][t];
      if (sspec[t] == sp && v == v) {
        const float lo = sul[j][t];
        if (kSum) s += (double)v + (double)lo;
        const long long key = ff_key(v, lo);
        mn = min(mn, key);
        mx = max(mx, key);
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      if (kSum) s += __shfl_down_sync(0xffffffffu, s, off);
      mn = min(mn, __shfl_down_sync(0xffffffffu, mn, off));
      mx = max(mx, __shfl_down_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) {
      double* pt = a.part + (((size_t)(g0 + j) * A.ntile + tile) * A.numslv + (sp - 1)) * 3;
      pt[0] = s;
      reinterpret_cast<long long*>(pt)[1] = mn;  // kFfKeyNone: no molecule of the species
      reinterpret_cast<long long*>(pt)[2] = mx;
    }
  }
}

// Mixed path, step 2 -- per molecule x G placements: float-float sums of the site terms
// and of the real-space pair terms, the residual, then the G bin searches in lockstep
// (binary lifting over the float keys of the edges staged in shared memory, finished
// exactly against the FP64 edges), histograms and per-species partials.
template <int G>
__global__ void __launch_bounds__(256, 3) mol_finish_kernel(MolArgs A, const float* __restrict__ site_e) {
  extern __shared__ int smem_dyn[];
  // [G][ermax] block histograms, or none when they would not fit beside other blocks: the
  // molecules' counts then go to the batch histograms in global memory (warp-aggregated).
  // Before the histograms are zeroed, the same region holds the FP64 pass's scratch
  // (finish_scratch_ints ints).
  int* smem_hist = A.hist_global ? nullptr : smem_dyn;
  int* skeys = smem_dyn + finish_region_ints(G, A.ermax, A.hist_global);  // [ermax] 32-bit edge keys
  int* sitem = smem_dyn;                                                     // [256][kBigPerThread]
  unsigned short* slist = reinterpret_cast<unsigned short*>(sitem + 256 * kBigPerThread);
  int* ss0 = reinterpret_cast<int*>(slist + 256 * kBigPerThread);           // [256]
  double* sbuf = reinterpret_cast<double*>(ss0 + 256);                      // [256]
  __shared__ int swarp[8];
  __shared__ float su[G][256];   // totals, hi part (NaN: no molecule)
  __shared__ float sul[G][256];  // totals, lo part
  __shared__ float sres[G];      // residual factor x solute charge of the G placements
  __shared__ float srcut[G];     // bounding-sphere cutoff of the real-space sum
  __shared__ int skskip[G];      // slot of the solute molecule itself (not a solvent)
  __shared__ int srej[G];        // placement rejected by check_mol_configuration
  __shared__ int4 supos[G];      // first solute site (fixed point)
  __shared__ unsigned char sspec[256];
  const int tile = blockIdx.y;
  const int g0 = blockIdx.x * G;
  const BatchArgs& a = A.a;
  const int ng = min(G, a.nb - g0);
  const int m = tile * blockDim.x + threadIdx.x;
  const bool valid = m < A.slvmax;
  for (int i = threadIdx.x; i < A.ermax; i += blockDim.x) skeys[i] = A.uvkey_f[i];
  if (threadIdx.x < ng) {
    const int b = g0 + threadIdx.x;
    sres[threadIdx.x] = (float)(A.resid_fac * a.u_qmol[b]);
    srcut[threadIdx.x] = A.rc_f + a.u_radius[b] + A.frame_scal[0];
    const int tg = a.tagslt[b] - 1;
    skskip[threadIdx.x] = (tg >= 0 && tg < A.nummol) ? A.mol_to_k[tg] : -2;
    srej[threadIdx.x] = (a.skip && a.skip[b]) ? 1 : 0;
    supos[threadIdx.x] = a.u_pos[(size_t)b * kMaxSoluteSites];
  }
  int k = -1, s0 = 0, ns = 0, species = 0;
  // residual_ene's molecular charge: the term pi Q_u Q_v / (beta^2 V) is below 1e-2 kcal/mol
  // for unit charges in these boxes, so its FP32 product is exact to 1e-9 kcal/mol
  float qmol = 0.f;
  if (valid) {
    k = A.slot_mol[m];
    s0 = A.slot_site[m];
    ns = A.slot_site[m + 1] - s0;
    species = A.slot_species[m];
    qmol = (float)A.slot_qmol[m];
  }
  const bool spec_ok = valid && species >= 1 && species <= A.numslv;
  sspec[threadIdx.x] = (unsigned char)(spec_ok ? species : 0);
  const int ldb = A.ldb;
  const LjK& k32 = A.k32;
  int sp_off = 0, sp_n = 1, sp_soft = 1;
  if (spec_ok) {
    sp_off = A.spec[3 * (species - 1)];
    sp_n = A.spec[3 * (species - 1) + 1];
    sp_soft = A.spec[3 * (species - 1) + 2];
  }
  __syncthreads();  // sres staged
  // ---- totals of the G placements, as float-float numbers.  First the site terms: the G
  // placements' terms of a site are G consecutive floats (16-byte loads when G, g0 and ldb
  // are multiples of 4).  The totals then wait in this thread's entries of su (hi) and sul
  // (lo) until the bin search; the real-space pass adds to them placement by placement in a
  // rolled loop (one copy of its code) ----
  unsigned actm = 0u;  // placements whose total is a solvent molecule's energy
  unsigned fix = 0u;   // placements with pairs left for the FP64 pass
  int nbig = 0;        // such pairs of this thread (the first kBigPerThread recorded in sitem)
  int* items = sitem + threadIdx.x * kBigPerThread;
  {
    ff rs[G];
#pragma unroll
    for (int j = 0; j < G; ++j) rs[j] = ff{0.f, 0.f};
    if (valid) {
      for (int s = 0; s < (A.bare ? 0 : ns); ++s) {
        const float* row = site_e + (size_t)(s0 + s) * ldb + g0;
        if (G % 4 == 0 && ng == G) {
#pragma unroll
          for (int j4 = 0; j4 < G; j4 += 4) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(row + j4));
            rs[j4] = ff_add(rs[j4], v.x);
            rs[j4 + 1] = ff_add(rs[j4 + 1], v.y);
            rs[j4 + 2] = ff_add(rs[j4 + 2], v.z);
            rs[j4 + 3] = ff_add(rs[j4 + 3], v.w);
          }
        } else {
#pragma unroll
          for (int j = 0; j < G; ++j)
            if (j < ng) rs[j] = ff_add(rs[j], __ldg(row + j));
        }
      }
    }
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const bool on = j < ng && valid && k != skskip[j] && !srej[j];
      if (on) actm |= 1u << j;
      // residual_ene (engproc.F90:859-869)
      const ff t = on ? ff_add(rs[j], -sres[j] * qmol) : ff{0.f, 0.f};
      su[j][threadIdx.x] = t.hi;
      sul[j][threadIdx.x] = t.lo;
    }
  }
  const int4 p0 = valid ? A.site_pos[s0] : make_int4(0, 0, 0, 0);
#pragma unroll 1
  for (int j = 0; j < G; ++j) {
    if (!(actm & (1u << j))) continue;
    // get_uv_energy (engproc.F90:736-753): real + residual + recip
    const ff r = real_mixed<true>(A, a, g0 + j, s0, ns, k32, srcut[j], p0, supos[j], j, items, 0, nbig, fix);
    if (r.hi != 0.f || r.lo != 0.f) {
      const ff t = ff_add2(ff{su[j][threadIdx.x], sul[j][threadIdx.x]}, r);
      su[j][threadIdx.x] = t.hi;
      sul[j][threadIdx.x] = t.lo;
    }
  }
  // ---- FP64 pass over the pair parts left out above (overlapping pairs).  The block's
  // recorded pairs are compacted (an exclusive scan over the threads) and evaluated one
  // per thread, so that every FP64 instruction of the pass runs on full warps; each owner
  // then adds its pairs' values in the order it found them.  A thread with more than
  // kBigPerThread pairs takes further rounds, recording the next ones by a fresh scan. ----
  if (__syncthreads_or(fix != 0u)) {
    ss0[threadIdx.x] = s0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int win = 0;; win += kBigPerThread) {
      if (win > 0) {  // later round: record pairs win .. win + kBigPerThread - 1 afresh
        int n2 = 0;
        unsigned f2 = 0u;
        if (nbig > win)
          for (int j = 0; j < G; ++j)
            if (fix & (1u << j)) real_mixed<false>(A, a, g0 + j, s0, ns, k32, srcut[j], p0, supos[j], j, items, win, n2, f2);
      }
      const int cnt = min(max(nbig - win, 0), kBigPerThread);
      // exclusive scan of cnt over the block
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      if (lane == 31) swarp[wid] = incl;
      __syncthreads();
      int off = incl - cnt, total = 0;
      for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) {
        if (w2 < wid) off += swarp[w2];
        total += swarp[w2];
      }
      if (total == 0) break;  // block-uniform
      for (int i = 0; i < cnt; ++i) slist[off + i] = (unsigned short)(threadIdx.x * kBigPerThread + i);
      __syncthreads();
      for (int base = 0; base < total; base += blockDim.x) {
        const int q = base + threadIdx.x;
        double v = 0.0;
        if (q < total) {
          const int slot = slist[q];
          const int t = slot / kBigPerThread, it = sitem[slot];
          const int j = (it >> 21) & 7, su_ = (it >> 13) & 0xff, sv = it & 0x1fff;
          const size_t us = (size_t)(g0 + j) * kMaxSoluteSites + su_;
          v = pair_fp64(A, ss0[t] + sv, a.u_x + us * 3, a.u_q[us], a.u_pos[us].w, it >> 24);
        }
        sbuf[threadIdx.x] = v;
        __syncthreads();
        for (int i = 0; i < cnt; ++i) {
          const int qq = off + i - base;
          if (qq < 0 || qq >= (int)blockDim.x) continue;
          const int j = (items[i] >> 21) & 7;
          const ff t = ff_add2(ff{su[j][threadIdx.x], sul[j][threadIdx.x]}, ff_from_double(sbuf[qq]));
          su[j][threadIdx.x] = t.hi;
          sul[j][threadIdx.x] = t.lo;
        }
        __syncthreads();
      }
    }
    __syncthreads();  // the scratch is free: the histograms may take the region
  }
  if (!A.hist_global)
    for (int i = threadIdx.x; i < G * A.ermax; i += blockDim.x) smem_hist[i] = 0;
  int ku[G];     // ordered key of the total's hi part
  float ulo[G];  // the total's lo part
#pragma unroll
  for (int j = 0; j < G; ++j) {
    ku[j] = ordered_key32(su[j][threadIdx.x]);
    ulo[j] = sul[j][threadIdx.x];
  }
  if (valid && a.uvengy_out) {
#pragma unroll
    for (int j = 0; j < G; ++j) {
      if (j >= ng) break;
      a.uvengy_out[(size_t)(a.b0 + g0 + j) * (A.slvmax + 1) + k + 1] =
          (actm & (1u << j)) ? (double)key32_to_float(ku[j]) + (double)ulo[j] : 0.0;
    }
  }
  __syncthreads();  // histograms zeroed, keys staged
  // ---- getiduv / binsearch for all G at once: pos = #edges whose float keys lie below
  // the key of the total's hi part ----
  int pos[G];
#pragma unroll
  for (int j = 0; j < G; ++j) pos[j] = 0;
  int step = 1;
  while ((step << 1) <= sp_n) step <<= 1;
  const int* kk = skeys + sp_off;
  for (; step > 0; step >>= 1) {
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const int q = pos[j] + step;
      if (q <= sp_n && kk[q - 1] < ku[j]) pos[j] = q;
    }
  }
#pragma unroll
  for (int j = 0; j < G; ++j) {
    float hv = __uint_as_float(0x7fc00000u);  // NaN marks "no molecule"
    float lv = 0.f;
    if (actm & (1u << j)) {
      const float v = key32_to_float(ku[j]), lo = ulo[j];
      int ret = pos[j];
      int code = 0;
      if (!spec_ok) {
        code = ERMOD_E_ENG_CNS;
      } else if (v != v) {
        code = ERMOD_E_ENG_MIN;
      } else {
        ret = exact_count(A.uvkey + sp_off, kk, sp_n, ret, ku[j], v, lo);
        if (ret <= 0)
          code = ERMOD_E_ENG_MIN;
        else if (A.soln && ret > sp_soft)
          code = ERMOD_E_ENG_SFT;
        else if (ret == sp_n && (v < 1.0e3f || (v == 1.0e3f && lo < 0.f)) && A.mbin_mode != 0) {
          if (A.mbin_mode == 1)
            code = ERMOD_W_MBIN;
          else
            atomicOr(&A.status->mbin_hit, 1);
        }
      }
      if (code)
        atomicMin(&A.status->err_key, make_err_key(a.b0 + g0 + j, k + 1, code));
      else
        hist_add(A.hist_global ? a.hist + (size_t)(g0 + j) * A.ermax : smem_hist + j * A.ermax, sp_off + ret - 1);
      if (a.mol_bin) a.mol_bin[(size_t)(g0 + j) * A.slvmax + m] = code ? A.ermax : sp_off + ret - 1;
      hv = v;
      lv = lo;
    } else if (a.mol_bin && valid && j < ng) {
      a.mol_bin[(size_t)(g0 + j) * A.slvmax + m] = A.ermax;
    }
    su[j][threadIdx.x] = hv;
    sul[j][threadIdx.x] = lv;
  }
  __syncthreads();
  // per-species {sum, min, max} of the block: one warp per (placement, species),
  // fixed lane order and a fixed shuffle tree; min and max as ordered keys of the
  // float-float totals (decoded by the reduce kernel), so that no FP64 instruction issues
  // here unless the species sums are wanted -- they are flceng (engproc.F90:822-825),
  // needed for slnuv (solution mode) and when the caller asks for flceng
  if (A.soln || a.flceng_out != nullptr)
    species_partials<G, true>(A, a, su, sul, sspec, g0, ng, tile);
  else
    species_partials<G, false>(A, a, su, sul, sspec, g0, ng, tile);
  if (A.hist_global) return;
  for (int j = 0; j < ng; ++j) {
    const int* h = smem_hist + j * A.ermax;
    int* out = a.hist + (size_t)(g0 + j) * A.ermax;
    for (int i = threadIdx.x; i < A.ermax; i += blockDim.x) {
      const int c = h[i];
      if (c) atomicAdd(out + i, c);
    }
  }
}

cudaError_t launch_p(Engine& e, const MolArgs& A, dim3 grid, size_t smem) {
  switch (e.P_order) {
    case 4:
      mol_energy_kernel<4><<<grid, 256, smem, A.a.stream>>>(A);
      break;
    case 6:
      mol_energy_kernel<6><<<grid, 256, smem, A.a.stream>>>(A);
      break;
    case 8:
      mol_energy_kernel<8><<<grid, 256, smem, A.a.stream>>>(A);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

static MolArgs make_mol_args(Engine& e, const BatchArgs& a) {
  MolArgs A{};
  A.site_pos = e.d_site_pos;
  A.site_rec = e.d_site_rec;
  A.site_grid = e.d_site_grid;
  A.site_x = e.d_site_x;
  A.site_w = e.d_site_w;
  A.site_q = e.d_site_q;
  A.slot_mol = e.d_slot_mol;
  A.slot_site = e.d_slot_site;
  A.slot_species = e.d_slot_species;
  A.slot_qmol = e.d_slot_qmol;
  A.frame_scal = e.d_frame_scal;
  A.mol_to_k = e.d_mol_to_k;
  A.slvmax = e.slvmax;
  A.nummol = e.nummol;
  A.ljene = e.d_ljene;
  A.ljlensq = e.d_ljlensq;
  A.ljene_f = e.d_ljene_f;
  A.ljlensq_f = e.d_ljlensq_f;
  A.T = e.ljtype_max;
  A.ldb = e.Bmax;
  A.uvkey = e.d_uvkey;
  A.uvkey_f = e.d_uvkey_f;
  // finish kernel: block histograms in shared memory up to 64 KB (three blocks per SM
  // fit); beyond that the counts go straight to global memory
  A.hist_global = (size_t)a.G * e.ermax * sizeof(int) > 64 * 1024 ? 1 : 0;
  A.spec = e.d_spec;
  A.numslv = e.numslv;
  A.ermax = e.ermax;
  A.soln = (e.P.slttype == 1) ? 1 : 0;
  A.mbin_mode = e.warn_bin_firsttime ? (e.P.force_calculation ? 2 : 1) : 0;
  A.g = e.geom;
  A.ljswitch = e.P.ljswitch;
  // non-periodic: the Coulomb cutoff is infinite (realcal.F90:174)
  A.elecut = e.geom.periodic ? e.P.elecut : HUGE_VAL;
  A.lwljcut = e.P.lwljcut;
  A.upljcut = e.P.upljcut;
  A.screen = e.P.screen;
  A.bare = (e.P.cltype == 0) ? 1 : 0;
  A.resid_fac = A.bare ? 0.0 : kPi / e.P.screen / e.P.screen / e.geom.volume;
  for (int i = 0; i < 3; ++i) A.fxf[i] = (float)e.geom.fx_scale[i];
  A.screen_f = (float)e.P.screen;
  A.rc_f = (float)std::max(A.elecut, e.P.upljcut);
  A.k64 = make_k64(A);
  A.k32 = to_f32(A.k64);
  A.a = a;
  A.ntile = e.ntile;
  A.status = e.d_status;
  return A;
}

// step 1 of the mixed path: gather by bricks (TMA-staged halos, double-buffered over
// placement groups) into a.site_e
cudaError_t launch_gather(Engine& e, const BatchArgs& a) {
  cudaError_t err = cudaSuccess;
  const int ngroups = (a.nb + 3) / 4;
  const int gpc = std::min(ngroups, 8);
  dim3 g1(e.nbricks, (ngroups + gpc - 1) / gpc);
  const int K1 = e.geom.K[0], K2 = e.geom.K[1], K3 = e.geom.K[2];
  const size_t npt = (size_t)e.gbox[0] * e.gbox[1] * e.gbox[2];
  const size_t hstride = (npt + 7) & ~(size_t)7;  // as in the kernel: 128-byte aligned halos
  const size_t sh = 128 + kGatherStages * hstride * sizeof(float4);
#define ERMOD_GATHER(PP)                                                                                        \
  if (e.P_order == PP) {                                                                                        \
    static SmemAttr attr;                                                                                       \
    if ((err = attr.ensure(gather_tma_kernel<PP>, sh)) != cudaSuccess) return err;                              \
    gather_tma_kernel<PP><<<g1, kGatherThreads, sh, a.stream>>>(                                                \
        e.phi_tmap[a.slot], a.nb, gpc, e.d_site_rec, e.d_site_grid, e.d_brick_site, e.d_brick_start, K1, K2, K3,  \
        e.nbrick[0], e.nbrick[1], e.gbox[0], e.Bmax, a.site_e, e.d_status);                                     \
  }
  ERMOD_GATHER(4)
  ERMOD_GATHER(6)
  ERMOD_GATHER(8)
#undef ERMOD_GATHER
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_mol_energy(Engine& e, const BatchArgs& a) {
  const MolArgs A = make_mol_args(e, a);
  const size_t smem = sizeof(int) * (size_t)a.G * e.ermax;
  dim3 grid(e.ntile, (a.nb + a.G - 1) / a.G);
  e.count_launch();
  cudaError_t err = cudaSuccess;
  if (!e.mixed) {
    static SmemAttr attr4, attr6, attr8;
    if ((err = attr4.ensure(mol_energy_kernel<4>, smem)) != cudaSuccess ||
        (err = attr6.ensure(mol_energy_kernel<6>, smem)) != cudaSuccess ||
        (err = attr8.ensure(mol_energy_kernel<8>, smem)) != cudaSuccess)
      return err;
    return launch_p(e, A, grid, smem);
  }
  if (a.G != 8 && a.G != 4) return cudaErrorInvalidValue;
  if (e.P.cltype != 0 && (err = launch_gather(e, a)) != cudaSuccess) return err;
  if (a.phases) {
    e.phase_end_on(a.stream);
    e.phase_begin_on(PH_MOL, a.stream);
  }
  // step 2: per-molecule totals and binning (histograms + edge keys in shared memory)
  const size_t smem_f = sizeof(int) * ((size_t)finish_region_ints(a.G, e.ermax, A.hist_global) + e.ermax);
  dim3 g2((a.nb + a.G - 1) / a.G, e.ntile);
#define ERMOD_FINISH(GG)                                                                                   \
  if (a.G == GG) {                                                                                         \
    static SmemAttr attr;                                                                                  \
    if ((err = attr.ensure(mol_finish_kernel<GG>, smem_f)) != cudaSuccess) return err;                     \
    mol_finish_kernel<GG><<<g2, 256, smem_f, a.stream>>>(A, a.site_e);                                   \
  }
  ERMOD_FINISH(4)
  ERMOD_FINISH(8)
#undef ERMOD_FINISH
  e.count_launch();
  return cudaGetLastError();
}


// ---- adjoint mode -------------------------------------------------------------------
//
// For a placement b of the differentiated solute and every solvent molecule k, the
// derivatives of u_k = real(k) + residual(k) + recip(k) (get_uv_energy,
// engproc.F90:662-756) with respect to each solute site's charge q_s (topology units),
// LJ epsilon eps_s and LJ sigma sigma_s:
//   du/dq_s     = sum_t q_t erfc(beta r)/r (r <= elecut) + sum_t q_t phi_s(r_t) - pi Q_k/(beta^2 V)
//   du/deps_s   = sum_t LJ_st / (2 eps_s)                       (eps_st = sqrt(eps_s eps_t))
//   du/dsigma_s = sum_t 4 eps_st (6 vdwa - 3 vdwb)/sigma_st^2 * d(sigma_st^2)/d(sigma_s)
// where phi_s is the PME potential of a unit charge on site s (computed by the mixed
// kernels as a batch of single-site "placements") and LJ_st = 4 eps_st (vdwa - vdwb) in
// every switching form (realcal.F90:686-770), vdwa ~ sigma^12 and vdwb ~ sigma^6.  Each
// molecule's derivatives (FP32) are then summed per energy bin of u_k in FP64, in a fixed
// order (molecules stably sorted by bin), times the placement's weight engnmfc.
namespace {

__device__ __forceinline__ void lj_parts_f(int sw, const LjK& k, float x, float r2, float& vdwa, float& vdwb) {
  const float invr2 = x / r2;
  const float invr6 = invr2 * invr2 * invr2;
  const float s6 = x * x * x;
  if (r2 <= k.lw2) {
    if (sw <= 1) {
      vdwa = invr6 * invr6;
      vdwb = invr6;
    } else if (sw == 2) {
      vdwa = invr6 * invr6 - s6 * s6 / (k.lw6 * k.up6);
      vdwb = invr6 - s6 / (k.lw3 * k.up3);
    } else {
      vdwa = invr6 * invr6 - s6 * s6 * k.repC;
      vdwb = invr6 - s6 * k.attC;
    }
    return;
  }
  if (sw == 0) {
    const float dd = r2 - k.up2, den = k.up2 - k.lw2;
    const float f = (2.f * r2 + k.up2 - 3.f * k.lw2) * (dd * dd) / (den * den * den);
    vdwa = invr6 * invr6 * f;
    vdwb = invr6 * f;
  } else if (sw == 1) {
    const float t = (sqrtf(r2) - k.lw) / (k.up - k.lw);
    const float t3 = t * t * t, t4 = t3 * t, t5 = t4 * t;
    const float f = 1.f - 10.f * t3 + 15.f * t4 - 6.f * t5;
    vdwa = invr6 * invr6 * f;
    vdwb = invr6 * f;
  } else if (sw == 2) {
    const float invr3 = sqrtf(invr6), s3 = sqrtf(s6);
    const float a = invr6 - s6 / k.up6, b = invr3 - s3 / k.up3;
    vdwa = k.up6 / (k.up6 - k.lw6) * (a * a);
    vdwb = k.up3 / (k.up3 - k.lw3) * (b * b);
  } else {
    const float f = sqrtf(r2) - k.lw;
    const float f3 = f * f * f, f4 = f3 * f;
    vdwa = invr6 * invr6 - s6 * s6 * (k.repA * f3 + k.repB * f4 + k.repC);
    vdwb = invr6 - s6 * (k.attA * f3 + k.attB * f4 + k.attC);
  }
}

struct AdjArgs {
  int b;          // placement within the batch
  int s_begin;    // first solute site of this chunk of unit-charge potentials
  int nchunk;     // sites in the chunk
  int nsu;        // solute sites: 3 nsu parameters
  int adj_mol;    // 1-based molecule whose placements are differentiated
  int cmbrule;
  int first;      // first chunk: also writes the bin keys
  const float* site_e_ps;  // [nsite][ldb] q_t phi_s(r_t) of the chunk's sites
  const int* mol_bin;      // [slvmax] bins of placement b's molecules, slot order (ermax: none)
  const float2* par;       // [nsu] {eps_s, sigma_s}
  float* du;               // [slvmax][3 nsu]
  int* key;                // [slvmax] global bin, or ermax to leave the molecule out
  int* val;                // [slvmax] slot index
};

__global__ void __launch_bounds__(256) adjoint_mol_kernel(MolArgs A, AdjArgs J) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= A.slvmax) return;
  const BatchArgs& a = A.a;
  const int b = J.b;
  const int k = A.slot_mol[m];
  const int s0 = A.slot_site[m];
  const int ns = A.slot_site[m + 1] - s0;
  const int species = A.slot_species[m];
  const int tg = a.tagslt[b] - 1;
  const int kskip = (tg >= 0 && tg < A.nummol) ? A.mol_to_k[tg] : -2;
  bool take = (tg + 1 == J.adj_mol) && (k != kskip) && species >= 1 && species <= A.numslv &&
              !(a.skip && a.skip[b]);
  if (J.first) {
    // the molecule's bin as the finish kernel found it (ermax: not binned)
    const int key = take ? J.mol_bin[m] : A.ermax;
    J.key[m] = key;
    J.val[m] = m;
  }
  if (!take) return;
  const size_t ub = (size_t)b * kMaxSoluteSites;
  const int P = 3 * J.nsu;
  const float fx = A.fxf[0], fy = A.fxf[1], fz = A.fxf[2];
  const LjK& k32 = A.k32;
  const float beta = A.screen_f;
  const float rq = (float)A.resid_fac * (float)A.slot_qmol[m];
  // the molecule is near the solute when its first site lies within the solute's
  // bounding sphere plus the cutoff (the finish kernel's test)
  const int4 p0 = A.site_pos[s0];
  const int4 q0 = a.u_pos[ub];
  const float dx0 = (float)(int)((unsigned)p0.x - (unsigned)q0.x) * fx;
  const float dy0 = (float)(int)((unsigned)p0.y - (unsigned)q0.y) * fy;
  const float dz0 = (float)(int)((unsigned)p0.z - (unsigned)q0.z) * fz;
  const float rcut = A.rc_f + a.u_radius[b] + A.frame_scal[0];
  const bool near = dx0 * dx0 + dy0 * dy0 + dz0 * dz0 <= rcut * rcut;
  for (int j = 0; j < J.nchunk; ++j) {
    const int s = J.s_begin + j;
    float dq = -rq, deps = 0.f, dsig = 0.f;
    for (int t = 0; t < ns; ++t) dq += J.site_e_ps[(size_t)(s0 + t) * A.ldb + j];
    if (near) {
      const int4 up = a.u_pos[ub + s];
      const float2 par = J.par[s];
      for (int t = 0; t < ns; ++t) {
        const int4 vp = A.site_pos[s0 + t];
        const float ex = (float)(int)((unsigned)vp.x - (unsigned)up.x) * fx;
        const float ey = (float)(int)((unsigned)vp.y - (unsigned)up.y) * fy;
        const float ez = (float)(int)((unsigned)vp.z - (unsigned)up.z) * fz;
        const float r2 = ex * ex + ey * ey + ez * ez;
        const float ljeps = A.ljene_f[vp.w + A.T * up.w];
        if (ljeps > 0.f && r2 <= k32.up2) {
          const float x = A.ljlensq_f[vp.w + A.T * up.w];
          float va, vb;
          lj_parts_f(A.ljswitch, k32, x, r2, va, vb);
          if (par.x > 0.f) deps += 4.f * ljeps * (va - vb) / (2.f * par.x);
          const float dldx = 4.f * ljeps * (6.f * va - 3.f * vb) / x;
          const float dxds = (J.cmbrule == 0) ? sqrtf(x) : (par.y > 0.f ? x / par.y : 0.f);
          dsig += dldx * dxds;
        }
        if (r2 <= k32.ele2) {
          const float r = sqrtf(r2);
          dq += A.site_rec[s0 + t].w * erfcf(beta * r) / r;
        }
      }
    }
    float* o = J.du + (size_t)m * P + 3 * s;
    o[0] = dq;
    o[1] = deps;
    o[2] = dsig;
  }
}

// the chunk's unit-charge single-site placements: site s_begin + j of placement b
__global__ void adjoint_pseudo_kernel(const float2* __restrict__ bvec, int b, int s_begin, int Kmax, int* nsite,
                                      float* qf, float2* ps_bvec) {
  const int j = blockIdx.x;
  if (threadIdx.x == 0) {
    nsite[j] = 1;
    qf[(size_t)j * kMaxSoluteSites] = 1.f;
  }
  const float2* src = bvec + ((size_t)b * kMaxSoluteSites + s_begin + j) * 3 * Kmax;
  float2* dst = ps_bvec + (size_t)j * kMaxSoluteSites * 3 * Kmax;
  for (int i = threadIdx.x; i < 3 * Kmax; i += blockDim.x) dst[i] = src[i];
}

__global__ void adjoint_bounds_kernel(const int* __restrict__ key, int n, int ermax, int* seg_b, int* seg_e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int kk = key[i];
  if (kk >= ermax) return;
  if (i == 0 || key[i - 1] != kk) seg_b[kk] = i;
  if (i == n - 1 || key[i + 1] != kk) seg_e[kk] = i + 1;
}

// one CTA per bin, one thread per parameter: FP64 sums in the sorted (bin, slot) order
__global__ void adjoint_reduce_kernel(const int* __restrict__ val, const float* __restrict__ du, int P,
                                      const int* __restrict__ seg_b, const int* __restrict__ seg_e,
                                      const double* __restrict__ engnmfc, int b, int ermax, double* grad,
                                      double* wsum) {
  const int bin = blockIdx.x;
  const int i0 = seg_b[bin], i1 = seg_e[bin];
  if (i0 >= i1) return;
  const double w = engnmfc[b];
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    double acc = 0.0;
    for (int i = i0; i < i1; ++i) acc += (double)du[(size_t)val[i] * P + p];
    grad[(size_t)p * ermax + bin] += w * acc;
  }
  if (threadIdx.x == 0) wsum[bin] += w * (double)(i1 - i0);
}

int key_bits(int ermax) {
  int bits = 1;
  while ((1 << bits) <= ermax) ++bits;
  return bits;
}

}  // namespace

size_t adjoint_cub_bytes(int n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (int*)nullptr, (int*)nullptr, (int*)nullptr, (int*)nullptr, n);
  return bytes;
}

cudaError_t launch_adjoint(Engine& e, const BatchArgs& a, cudaStream_t s) {
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const int n = e.slvmax;
  const int P = 3 * e.adj_ns;
  const int chunk = e.Bmax;
  int* key = e.d_adj_key;
  int* val = key + n;
  int* key_s = val + n;
  int* val_s = key_s + n;
  for (int b = 0; b < a.nb; ++b) {
    for (int s0 = 0; s0 < e.adj_ns; s0 += chunk) {
      const int nch = std::min(chunk, e.adj_ns - s0);
      adjoint_pseudo_kernel<<<nch, 128, 0, s>>>(a.u_bvec, b, s0, e.Kmax(), e.d_ps_nsite, e.d_ps_qf, e.d_ps_bvec);
      e.count_launch();
      BatchArgs pa = a;  // unit charges on single sites, this slot's grids and site terms
      pa.nb = nch;
      pa.u_nsite = e.d_ps_nsite;
      pa.u_qf = e.d_ps_qf;
      pa.u_bvec = e.d_ps_bvec;
      pa.self_part = e.d_ps_self;
      pa.stream = s;
      pa.phases = 0;
      if ((err = launch_pme_mixed(e, pa)) != cudaSuccess) return err;
      if ((err = launch_gather(e, pa)) != cudaSuccess) return err;
      MolArgs A = make_mol_args(e, a);
      AdjArgs J{};
      J.b = b;
      J.s_begin = s0;
      J.nchunk = nch;
      J.nsu = e.adj_ns;
      J.adj_mol = e.adj_mol;
      J.cmbrule = e.adj_cmbrule;
      J.first = (s0 == 0);
      J.site_e_ps = a.site_e;
      J.mol_bin = a.mol_bin + (size_t)b * n;
      J.par = e.d_adj_par;
      J.du = e.d_adj_du;
      J.key = key;
      J.val = val;
      adjoint_mol_kernel<<<(n + 255) / 256, 256, 0, s>>>(A, J);
      e.count_launch();
      if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    size_t bytes = e.adj_cub_bytes;
    err = cub::DeviceRadixSort::SortPairs(e.d_adj_cub, bytes, key, key_s, val, val_s, n, 0, key_bits(e.ermax), s);
    if (err != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(e.d_adj_seg, 0, sizeof(int) * 2 * (size_t)e.ermax, s)) != cudaSuccess) return err;
    adjoint_bounds_kernel<<<(n + 255) / 256, 256, 0, s>>>(key_s, n, e.ermax, e.d_adj_seg, e.d_adj_seg + e.ermax);
    adjoint_reduce_kernel<<<e.ermax, 64, 0, s>>>(val_s, e.d_adj_du, P, e.d_adj_seg, e.d_adj_seg + e.ermax, a.engnmfc,
                                                 b, e.ermax, e.d_adj_grad, e.d_adj_w);
    e.count_launch(2);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  return cudaSuccess;
}

}  // namespace ermod
