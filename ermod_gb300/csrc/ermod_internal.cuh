// ermod_internal.cuh -- device data layout and kernel launchers of the GB300 path.
//
// Data layout in HBM (one context):
//   topology   per-atom charge/ljtype, per physical molecule (tagpt order) species,
//              molecular charge and site range;
//   frame      raw sitepos (3, numatm) FP64; per physical site, in the frame's
//              spatially sorted molecule order ("slot" order):
//                pos   int4 {X, Y, Z, ljtype}  -- wrapped coordinates as 32-bit fixed
//                      point, X = x / L * 2^32 (periodic minimum image is an int32
//                      subtraction);
//                rec   float4 {t1, t2, t3, q}  -- B-spline fractional offsets and charge;
//                grid  int, packed base grid point g1 | g2 << 10 | g3 << 20;
//              wrapped FP64 coordinates and FP64 charge (both paths), FP64 spline
//              weights (FP64 path);
//   green      engfac[K3][K2][K1/2+1] FP64 (+ FP32 copy for the mixed path);
//   batch      per placement solute sites, 1-D structure-factor vectors, PME spectrum
//              and potential grids, per-placement energy histograms;
//   accum      edens, ecorr (+ int64 count mirror), eself, slnuv, minuv/maxuv, scalars.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace ermod {

constexpr int kMaxSoluteSites = 256;  // sites of one solute molecule
constexpr int kMaxSplineOrder = 8;
// batch slots: the buffers of a batch (solute data, PME grids, site terms) in flight at
// once; batches alternate between two streams and take the slots in turn, so a batch
// reuses the buffers of the batch three before it, whose accumulation is long done
constexpr int kBatchSlots = 3;
// batch streams: batches take them in turn (batch i: stream i mod 2).  A third one was
// measured: +0.5% on the 96^3 workload and -2.4% at 48^3, with each kernel's in-pipeline
// launch time half as long again (it shares the SMs with two other batches)
constexpr int kBatchStreams = 2;
constexpr int kMaxSpecies = 16;
constexpr int kGridBits = 10;         // packed grid coordinates: K <= 1024 per axis
constexpr double kPi = 3.1415926535897932;

// B-spline weights M_P(t + j), j = 0..P-1, by the stable Cox-de Boor recursion (FP32)
template <int P>
__host__ __device__ __forceinline__ void bspline_w(float t, float w[P]) {
  w[0] = t;
  w[1] = 1.f - t;
#pragma unroll
  for (int j = 2; j < P; ++j) w[j] = 0.f;
#pragma unroll
  for (int n = 3; n <= P; ++n) {
    const float inv = 1.f / (float)(n - 1);
#pragma unroll
    for (int j = n - 1; j >= 0; --j) {
      const float a = (j <= n - 2) ? w[j] : 0.f;
      const float b = (j >= 1) ? w[j - 1] : 0.f;
      w[j] = ((t + (float)j) * a + ((float)n - t - (float)j) * b) * inv;
    }
  }
}

// Float-float numbers: the value hi + lo with |lo| <= ulp(hi) / 2, about 48 significant
// bits from FP32 operations only (Knuth's TwoSum, then a renormalisation).  The sums of
// the mixed path's per-molecule energies use them, so that the total that decides a bin
// carries no FP32 rounding of its own and no FP64 instruction is issued per molecule.
struct ff {
  float hi, lo;
};
__host__ __device__ __forceinline__ ff ff_add(ff a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b - bb);
  const float lo = a.lo + err;
  const float hi = s + lo;
  return ff{hi, lo - (hi - s)};
}
__host__ __device__ __forceinline__ ff ff_add2(ff a, ff b) { return ff_add(ff_add(a, b.hi), b.lo); }
// a double as a float-float (exact to 48 bits: hi = rn(d), lo = rn(d - hi))
__host__ __device__ __forceinline__ ff ff_from_double(double d) {
  const float hi = (float)d;
  return ff{hi, (float)(d - (double)hi)};
}
__host__ __device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// error key: (placement << 36) | (molecule << 8) | code, minimised atomically so the
// first failing (placement, molecule) in reference order wins.
constexpr unsigned long long kNoError = ~0ull;
__host__ __device__ inline unsigned long long make_err_key(int placement, int molecule, int code) {
  return ((unsigned long long)placement << 36) | ((unsigned long long)(molecule & 0x0fffffff) << 8) |
         (unsigned long long)(code & 0xff);
}

// ordered 64-bit key of a double (total order equal to numeric order, -0 == +0)
__host__ __device__ inline long long ordered_key(double x) {
  if (x == 0.0) x = 0.0;
  long long k;
#ifdef __CUDA_ARCH__
  k = __double_as_longlong(x);
#else
  __builtin_memcpy(&k, &x, 8);
#endif
  return k ^ ((k >> 63) & 0x7fffffffffffffffll);
}

// The dynamic shared memory a kernel may use, raised with cudaFuncSetAttribute when a
// launch needs more than before.  The attribute belongs to the device current at the call,
// so the largest size set so far is kept per device (contexts of one process may sit on
// several devices and several host threads).
struct SmemAttr {
  static constexpr int kMaxDevices = 64;
  std::atomic<size_t> set[kMaxDevices];
  template <typename F>
  cudaError_t ensure(F* f, size_t bytes) {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    const bool cached = dev >= 0 && dev < kMaxDevices;
    size_t cur = cached ? set[dev].load() : 0;
    if (cached && cur >= bytes) return cudaSuccess;
    err = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (err == cudaSuccess && cached)
      while (cur < bytes && !set[dev].compare_exchange_weak(cur, bytes)) {
      }
    return err;
  }
};

// bricks of the mixed path's gather: kBrickX x kBrickY x kBrickZ PME grid points
constexpr int kBrickX = 16, kBrickY = 8, kBrickZ = 8;

// ordered 32-bit key of a float (-0 == +0).  For a float u and a double edge e,
// u <= e exactly when u <= rd(e), the largest float not above e, and u > e exactly when
// u > rd(e); so a search of the keys of rd(edges) with the key of a float-float total's
// hi part finds its bin up to the edges within one float step of hi, which the finish
// kernel then compares exactly.
__host__ __device__ inline int ordered_key32(float f) {
  if (f == 0.0f) f = 0.0f;
  int k;
#ifdef __CUDA_ARCH__
  k = __float_as_int(f);
#else
  __builtin_memcpy(&k, &f, 4);
#endif
  return k ^ ((k >> 31) & 0x7fffffff);
}

#ifdef __CUDACC__
// float of an ordered 32-bit key (the inverse of ordered_key32)
__device__ __forceinline__ float key32_to_float(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); }

// ordered 64-bit key of a float-float number (hi, lo): hi first, then lo; the order of
// the keys is the order of the values hi + lo.  The mixed finish kernel keeps its
// per-species minimum and maximum energies as such keys; the reduce kernel decodes them.
__device__ __forceinline__ long long ff_key(float hi, float lo) {
  return (long long)(((unsigned long long)(unsigned)ordered_key32(hi) << 32) |
                     (unsigned long long)((unsigned)ordered_key32(lo) ^ 0x80000000u));
}
constexpr long long kFfKeyNone = 0x7fffffffffffffffll;        // min over no molecule
constexpr long long kFfKeyNoneMax = (long long)0x8000000000000000ull;  // max over no molecule
__device__ __forceinline__ double ff_key_to_double(long long k) {
  if (k == kFfKeyNone) return HUGE_VAL;
  if (k == kFfKeyNoneMax) return -HUGE_VAL;
  const float hi = key32_to_float((int)(k >> 32));
  const float lo = key32_to_float((int)((unsigned)k ^ 0x80000000u));
  return (double)hi + (double)lo;
}
#endif

struct FrameGeom {
  double L[3];       // cell lengths (cuboid cell)
  double invL[3];    // 1 / L as dtrtri computes it
  double invcl[9];   // engproc.F90:898-919, column-major
  double volume;
  double fx_scale[3];  // L / 2^32 (fixed point -> Angstrom)
  int K[3];
  // boxshp: 1 periodic; 0 non-periodic (realcal.F90:174,202): coordinates are not wrapped
  // and distances take no minimum image.  L is then a virtual cube for the fixed-point
  // coordinates and the spatial sort, large enough that no pair difference wraps, and
  // every solute coordinate must satisfy |x| < reach.
  int periodic;
  double reach;
};

// Device status block (one per context).  The host API resets it at every call; the
// device API keeps it across calls until ermod_sync reads and resets it.
struct DevStatus {
  unsigned long long err_key;    // first error of the current call (kNoError when none)
  unsigned long long first_key;  // device API: first error of an earlier call since the last sync
  int mbin_hit;                  // 'mbin' condition met (reported once)
  int range_fault;               // an index check failed on the device
};

// One batch of placements, as seen by the kernels.
struct BatchArgs {
  int nb;             // placements in this batch
  int b0;             // index of the batch's first placement within the call
  int G;              // placements per mol_energy block
  int n_u_max;        // max solute sites in the batch
  int slot;           // batch slot (batch index mod kBatchSlots): selects the PME grids' set
  cudaStream_t stream;  // stream of the batch's PME, gather and finish kernels
  float* site_e;      // [nsite_phys][Bmax] reciprocal site terms of this slot (mixed)
  int phases;         // 1: the launchers split the caller's timing phase (gather/finish...)
  int* mol_bin;       // [nb][slvmax] bin (0-based) of each molecule in slot order, ermax when
                      // not binned (adjoint mode), or null
  const int* tagslt;  // [nb] 1-based
  const double* stat_weight_solute;  // [nb] or null
  // solute site data per placement, [nb][kMaxSoluteSites]
  int* u_nsite;        // [nb]
  double* u_x;         // [nb][S][3] wrapped FP64 coords
  int4* u_pos;         // [nb][S] fixed point + ljtype
  double* u_q;         // [nb][S]
  float* u_qf;         // [nb][S] FP32 copy for the mixed kernels
  int* u_grid;         // [nb][S] packed base grid
  double* u_w;         // [nb][S][3][P] FP64 spline weights
  float2* u_bvec;      // [nb][S][3][Kmax] 1-D structure factors (mixed)
  double* u_qmol;      // [nb] molecular charge of the solute
  double* u_usreal;    // [nb] realcal_self value
  float* u_radius;     // [nb] solute bounding radius about site 1 (A)
  // PME
  float2* spec;        // [nb][K3][K2][H] mixed spectrum (engfac * S)
  float* phi;          // [nb][K3][K2][K1] mixed potential
  double2* spec64;     // FP64 path
  double* phi64;       // FP64 path
  double* self_part;   // [nb][K2] (mixed) or [nb][influence64_blocks] (FP64) partial self energies
  // outputs
  int* hist;           // [nb][ermax] instantaneous histogram (insdst)
  double* part;        // [nb][ntile][numslv][3] {sum, min, max}
  double* uvengy_out;  // [nplace][slvmax+1] or null (device)
  double* flceng_out;  // [nplace][numslv] or null (device)
  double* engnmfc;     // [nb] weights (0 for skipped placements)
  double* u0;          // [nb] solute self energies
  int* self_bin;       // [nb] eself bin (0-based) or -1
  const int* skip;     // [nb] 1: the configuration check skips the placement (solution mode), or null
};

struct Engine;

// ---- launchers (defined in the .cu files) ---------------------------------------
// frame preparation
cudaError_t launch_frame_wrap(Engine& e);
cudaError_t launch_carry_status(Engine& e);  // device API: an earlier call's error stops this call
cudaError_t launch_max_abs(Engine& e, const double* x_d, size_t n, double* host_out);  // syncs e.stream
cudaError_t launch_frame_sort(Engine& e);
cudaError_t launch_frame_sites(Engine& e);
cudaError_t launch_greenfunc(Engine& e);
// solution mode: the placements check_mol_configuration would skip (e.d_skip[0..nplace))
cudaError_t launch_config_check(Engine& e, int nplace, const int* d_tag);
// placement preparation and PME
cudaError_t launch_place_prep(Engine& e, const BatchArgs& a, const double* sol_xyz, int self_first_only,
                              cudaStream_t s);
cudaError_t launch_pme_mixed(Engine& e, const BatchArgs& a);
bool pme_fits(int K1, int K2, int K3);
cudaError_t launch_spread64(Engine& e, const BatchArgs& a);
cudaError_t launch_influence64(Engine& e, const BatchArgs& a);
// per-molecule energies and histograms
cudaError_t launch_mol_energy(Engine& e, const BatchArgs& a);
cudaError_t launch_gather(Engine& e, const BatchArgs& a);
// adjoint mode: bin-resolved solute-parameter derivatives of the batch's placements
cudaError_t launch_adjoint(Engine& e, const BatchArgs& a, cudaStream_t s);
size_t adjoint_cub_bytes(int n);
// device placements (kernels_insert.cu)
cudaError_t launch_insert(Engine& e, int nplace, int ns, const ermod_insert_params& ip, const double* bf_d,
                          const double* mass_d, double* out, double* weight);
// getsolute's structure window over the library: accepted structures to e.d_lib_acc
cudaError_t launch_library_filter(Engine& e, int insstructure, double lwstr, double upstr);
// accumulation
cudaError_t launch_accumulate(Engine& e, const BatchArgs& a, cudaStream_t s);
cudaError_t launch_ecorr_flush(Engine& e, cudaStream_t s);
// ecorr from caller histograms with the fixed scratch (no allocation); sizes checked by the caller
constexpr int kNoAllocMaxPlace = 4096;
constexpr int kNoAllocMaxBins = 8192;
constexpr long long kNoAllocMaxEntries = 1LL << 20;  // nplace * ermax
cudaError_t launch_ecorr_noalloc(const int* hist, const double* weight, int nplace, int ermax, double* ecorr,
                                 long long* ecorr_count, cudaStream_t s);

}  // namespace ermod
