// kernels_insert.cu -- test-particle placements generated on the device (instslt,
// insertion.F90:76-99: set_solute_origin, set_shift_com, apply_orientation).
//
// One thread per placement.  The reference draws from the Fortran compiler's
// random_number, a stream no other compiler reproduces, so the generator here is a
// counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): placement p of a
// call draws from counter (draw, offset + p) under key seed, so a placement's
// coordinates depend only on (seed, its global index) and not on thread order, batch
// size or device.  Uniform doubles take 53 bits from two 32-bit words.
//
// Modes (engmain.F90:320-326):
//   insorigin   0 COM to the origin, 1 as given, 2 COM to the host aggregate's centre,
//               3 best fit onto the reference solute carried into the frame (reffit)
//   insposition 0 random in the cell (COM = cell U^3), 1 as given, 2 spherical shell
//               lwreg..upreg about the origin, 3/4 slab (generic / symmetric) in z,
//               5 random translation within upreg + 3 x solute size, 6 uniform /
//               Gaussian mixture with its WHAM weight (insertion.F90:274-316)
//   insorient   0 rotation about the COM by a unit quaternion from rejection sampling
//               of U[-1,1]^4 (applied as q v q*, bestfit.F90:75-100), 1 none
// With insorigin 3 a placement whose RMSD from the fitted reference solute lies outside
// [lwreg, upreg] is drawn again (instslt's loop, insertion.F90:88-96, and
// check_solute_configuration, :569-595); as in the reference, the weight of insposition 6
// takes the factor of every draw, rejected ones included, and the uniform / Gaussian
// alternation advances per draw (draw d of placement g is uniform when g + d is even).
// A flexible solute (getsolute, insertion.F90:384-495) takes placement g's structure and
// initial weight from the structure library: the g-th accepted read of the wrapped file.
#include "bestfit.cuh"
#include "engine.cuh"

namespace ermod {

namespace {

struct Philox {
  uint32_t k0, k1;      // key
  uint32_t c2, c3;      // placement index (64-bit)
  uint32_t draw = 0;    // next 128-bit block
  uint32_t buf[4];
  int left = 0;

  __device__ __forceinline__ void block() {
    uint32_t c0 = draw++, c1 = 0, d2 = c2, d3 = c3, a = k0, b = k1;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
      const uint32_t hi1 = __umulhi(0xCD9E8D57u, d2), lo1 = 0xCD9E8D57u * d2;
      const uint32_t n0 = hi1 ^ c1 ^ a, n1 = lo1, n2 = hi0 ^ d3 ^ b, n3 = lo0;
      c0 = n0;
      c1 = n1;
      d2 = n2;
      d3 = n3;
      a += 0x9E3779B9u;
      b += 0xBB67AE85u;
    }
    buf[0] = c0;
    buf[1] = c1;
    buf[2] = d2;
    buf[3] = d3;
    left = 4;
  }
  __device__ __forceinline__ uint32_t u32() {
    if (left == 0) block();
    return buf[4 - left--];
  }
  __device__ __forceinline__ double uniform() {  // [0, 1), 53 bits
    const uint32_t a = u32() >> 5, b = u32() >> 6;
    return ((double)a * 67108864.0 + (double)b) * (1.0 / 9007199254740992.0);
  }
};

struct InsArgs {
  int nplace, ns;
  int insposition, insorient, insorigin;
  double lwreg, upreg;
  uint32_t k0, k1;
  unsigned long long offset;
  double cell[9];  // column major: cell(:, j) is the j-th cell vector
  const double* bf;    // [ns][3] reference solute coordinates
  const double* mass;  // [ns]
  double* out;         // [nplace][ns][3]
  double* weight;      // [nplace] or null
  const double* fit;   // insorigin 2: [3] aggregate centre; 3: [ns][3] origin, [ns][3] fitted reference
  const double* rw;    // insorigin 3: [ns][4] reference solute (weights at [4 s + 3])
  // flexible solute: structures [nconf][ns][3] (null: the rigid bf), weights [nwt] (nwt 0:
  // 1), the na accepted structures in file order
  const double* lib;
  const double* lib_wt;
  const int* lib_acc;
  int lib_nconf, lib_nwt, lib_na;
  DevStatus* status;
};

// redraws of one placement under the RMSD acceptance before it is reported as impossible
constexpr int kMaxRedraw = 1 << 16;

// rejection draws per loop; a loop that runs out (probability below 1e-40 for the
// quaternion, whose acceptance is pi^2/32) keeps its last draw
constexpr int kMaxTries = 256;

__device__ void com_of(const double* x, const double* m, int ns, double c[3]) {
  double w = 0.0;
  c[0] = c[1] = c[2] = 0.0;
  for (int s = 0; s < ns; ++s) {
    w += m[s];
    for (int i = 0; i < 3; ++i) c[i] += m[s] * x[3 * s + i];
  }
  for (int i = 0; i < 3; ++i) c[i] /= w;
}

__global__ void __launch_bounds__(128) insert_kernel(InsArgs A) {
  extern __shared__ double sh[];
  double* sbf = sh;                      // [ns][3]
  double* sm = sh + 3 * (size_t)A.ns;    // [ns]
  for (int i = threadIdx.x; i < 3 * A.ns; i += blockDim.x) sbf[i] = A.bf[i];
  for (int i = threadIdx.x; i < A.ns; i += blockDim.x) sm[i] = A.mass[i];
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= A.nplace) return;
  const unsigned long long g = A.offset + (unsigned long long)p;
  Philox rng;
  rng.k0 = A.k0;
  rng.k1 = A.k1;
  rng.c2 = (uint32_t)g;
  rng.c3 = (uint32_t)(g >> 32);
  double* x = A.out + (size_t)p * A.ns * 3;
  double weight = 1.0;
  const double* conf = sbf;  // bfcoord
  if (A.lib) {
    // getsolute: the g-th accepted read is read r = (g / na) nconf + acc[g mod na] of the
    // wrapped structure file; the weight file, read once per structure read, wraps on its own
    const unsigned long long na = (unsigned long long)A.lib_na;
    const int f = A.lib_acc[g % na];
    const unsigned long long r = (g / na) * (unsigned long long)A.lib_nconf + (unsigned long long)f;
    conf = A.lib + (size_t)f * A.ns * 3;
    if (A.lib_nwt > 0) weight = A.lib_wt[r % (unsigned long long)A.lib_nwt];
  }
  // set_solute_origin: bfcoord, or with insorigin 3 bfcoord fitted onto the reference
  // solute in the frame (once per call for a rigid solute, per placement for a library's)
  const bool refit = A.insorigin == 3 && A.lib;
  double fc1[3], fc2[3], fq[4];
  if (refit) {
    const double* best = A.fit + 3 * (size_t)A.ns;
    const double* rw = A.rw;
    bestfit::fit_transform(
        A.ns, [best](int s, int c) { return best[3 * s + c]; }, [conf](int s, int c) { return conf[3 * s + c]; },
        [rw](int s) { return rw[4 * s + 3]; }, fc1, fc2, fq);
  }
  const double* x0 = (A.insorigin == 3) ? A.fit : conf;
  double c[3];
  bool ok = true;  // every rejection loop accepted
  for (int draw = 0;; ++draw) {
    if (refit)
      for (int s = 0; s < A.ns; ++s) bestfit::apply_fit(fc1, fc2, fq, conf + 3 * s, x + 3 * s);
    else
      for (int i = 0; i < 3 * A.ns; ++i) x[i] = x0[i];
    if (A.insorigin == 0 || A.insorigin == 2) {  // set_solute_com(insml, 0 or the aggregate centre)
      com_of(x, sm, A.ns, c);
      for (int i = 0; i < 3; ++i) c[i] -= (A.insorigin == 2) ? A.fit[i] : 0.0;
      for (int s = 0; s < A.ns; ++s)
        for (int i = 0; i < 3; ++i) x[3 * s + i] -= c[i];
    }
    double shift[3] = {0.0, 0.0, 0.0};
    const double* C = A.cell;
    auto cell_times = [&](const double r[3], double out[3]) {  // matmul(cell, r)
      for (int i = 0; i < 3; ++i) out[i] = C[i] * r[0] + C[i + 3] * r[1] + C[i + 6] * r[2];
    };
    switch (A.insposition) {
      case 0: {  // COM to cell . U^3
        double r[3], t[3];
        for (int i = 0; i < 3; ++i) r[i] = rng.uniform();
        cell_times(r, t);
        com_of(x, sm, A.ns, c);
        for (int i = 0; i < 3; ++i) shift[i] = t[i] - c[i];
        break;
      }
      case 2: {  // spherical shell
        double t = rng.uniform();
        const double lw3 = A.lwreg * A.lwreg * A.lwreg, up3 = A.upreg * A.upreg * A.upreg;
        t = cbrt(t * (up3 - lw3) + lw3);
        double r[3], norm = 0.0;
        ok = false;
        for (int it = 0; it < kMaxTries && !ok; ++it) {
          for (int i = 0; i < 3; ++i) r[i] = rng.uniform() * 2.0 - 1.0;
          norm = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
          ok = (0.0 < norm) && (norm <= 1.0);
        }
        norm = sqrt(norm);
        for (int i = 0; i < 3; ++i) shift[i] = t * r[i] / norm;
        break;
      }
      case 3:
      case 4: {  // slab in z
        double r[3];
        r[0] = rng.uniform();
        r[1] = rng.uniform();
        double t = rng.uniform();
        t = t * (A.upreg - A.lwreg) + A.lwreg;
        if (A.insposition == 4) {
          const double dir = rng.uniform();
          if (dir > 0.5) t = -t;
        }
        const double celllen3 = sqrt(C[6] * C[6] + C[7] * C[7] + C[8] * C[8]);
        r[2] = t / celllen3;
        cell_times(r, shift);
        break;
      }
      case 5: {  // translation within upreg + 3 x (largest COM distance)
        com_of(x, sm, A.ns, c);
        double maxdis = 0.0;
        for (int s = 0; s < A.ns; ++s) {
          double d = 0.0;
          for (int i = 0; i < 3; ++i) d += (x[3 * s + i] - c[i]) * (x[3 * s + i] - c[i]);
          maxdis = fmax(maxdis, d);
        }
        const double movmax = A.upreg + 3.0 * sqrt(maxdis);
        for (int i = 0; i < 3; ++i) shift[i] = movmax * (2.0 * rng.uniform() - 1.0);
        break;
      }
      case 6: {  // uniform / Gaussian mixture, alternating over the global placement index
        double ls[3];
        for (int i = 0; i < 3; ++i) {
          const double len = sqrt(C[3 * i] * C[3 * i] + C[3 * i + 1] * C[3 * i + 1] + C[3 * i + 2] * C[3 * i + 2]);
          ls[i] = (len / 2.0) / A.upreg;
        }
        const double z0 = 8.0 * ls[0] * ls[1] * ls[2];
        const double sqpi = sqrt(3.14159265358979323846);
        const double z1 = sqpi * sqpi * sqpi * erf(ls[0]) * erf(ls[1]) * erf(ls[2]);
        double sc[3];
        if (((g + (unsigned long long)draw) & 1ull) == 0ull) {  // the reference starts with the uniform draw
          for (int i = 0; i < 3; ++i) sc[i] = (2.0 * rng.uniform() - 1.0) * ls[i];
        } else {
          for (int i = 0; i < 3; ++i) {
            double r = 0.0;
            bool in = false;
            for (int it = 0; it < kMaxTries && !in; ++it) {
              const double r1 = 1.0 - rng.uniform(), r2 = rng.uniform();  // nrand: Box-Muller on (0,1]
              r = sqrt(-2.0 * log(r1)) * cos(2.0 * 3.14159265358979323846 * r2) / sqrt(2.0);
              in = fabs(r) < ls[i];
            }
            ok = ok && in;
            sc[i] = r;
          }
        }
        const double sqsum = sc[0] * sc[0] + sc[1] * sc[1] + sc[2] * sc[2];
        weight = weight / (0.5 * 1.0 / z0 + 0.5 * exp(-sqsum) / z1);
        double r[3];
        for (int i = 0; i < 3; ++i) r[i] = sc[i] / (ls[i] * 2.0);
        cell_times(r, shift);
        break;
      }
      default:  // 1: as given
        break;
    }
    for (int s = 0; s < A.ns; ++s)
      for (int i = 0; i < 3; ++i) x[3 * s + i] += shift[i];
    if (A.insorient == 0) {  // rotate about the COM
      double q[4], n2 = 0.0;
      bool got = false;
      for (int it = 0; it < kMaxTries && !got; ++it) {
        for (int i = 0; i < 4; ++i) q[i] = rng.uniform() * 2.0 - 1.0;
        n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        got = n2 < 1.0;
      }
      ok = ok && got;
      const double inv = 1.0 / sqrt(n2);
      for (int i = 0; i < 4; ++i) q[i] *= inv;
      com_of(x, sm, A.ns, c);
      for (int s = 0; s < A.ns; ++s) {  // v' = v + w t + u x t, t = 2 u x v
        const double v[3] = {x[3 * s] - c[0], x[3 * s + 1] - c[1], x[3 * s + 2] - c[2]};
        const double t[3] = {2.0 * (q[2] * v[2] - q[3] * v[1]), 2.0 * (q[3] * v[0] - q[1] * v[2]),
                             2.0 * (q[1] * v[1] - q[2] * v[0])};
        x[3 * s + 0] = v[0] + q[0] * t[0] + (q[2] * t[2] - q[3] * t[1]) + c[0];
        x[3 * s + 1] = v[1] + q[0] * t[1] + (q[3] * t[0] - q[1] * t[2]) + c[1];
        x[3 * s + 2] = v[2] + q[0] * t[2] + (q[1] * t[1] - q[2] * t[0]) + c[2];
      }
    }
    if (A.insorigin != 3) break;
    // check_solute_configuration: rmsd_nofit(refslt_bestfit, the placement, refslt_weight)
    {
      const double* ref = A.fit + 3 * (size_t)A.ns;
      double W = 0.0, disp = 0.0;
      for (int s = 0; s < A.ns; ++s) {
        double d2 = 0.0;
        for (int i = 0; i < 3; ++i) d2 += (x[3 * s + i] - ref[3 * s + i]) * (x[3 * s + i] - ref[3 * s + i]);
        W += A.rw[4 * s + 3];
        disp += A.rw[4 * s + 3] * d2;
      }
      const double rmsd = sqrt(disp / W);
      if (!(A.lwreg > rmsd || rmsd > A.upreg)) break;
    }
    if (draw + 1 >= kMaxRedraw) {  // the region admits (almost) nothing: report it
      atomicMin(&A.status->err_key, make_err_key(p, 0, ERMOD_E_INS_GEO));
      break;
    }
  }
  (void)ok;
  if (A.weight) A.weight[p] = weight;
}

// The frame-wide part of set_solute_origin, one CTA: insorigin 2, the host aggregate's
// centre of mass (com_aggregate, insertion.F90:539-566) to fit[0..2]; insorigin 3,
// reffit (insertion.F90:598-624): the reference host fitted onto the frame's refspec
// atoms carries the reference solute into the frame (fit[3 ns ..]), and bfcoord fitted
// onto that is the placements' starting structure (fit[0 .. 3 ns)).  FP64.
__global__ void __launch_bounds__(256) insert_origin_kernel(const double* __restrict__ pos,
                                                            const double* __restrict__ agg_mass, int numatm,
                                                            int origin, const int* __restrict__ ref_atoms, int nh,
                                                            const double* __restrict__ ref_host,
                                                            const double* __restrict__ ref_slt, int ns,
                                                            const double* __restrict__ bf, double* __restrict__ fit) {
  __shared__ double red[9][256];
  auto reduce = [&](double* v, int n) {
    for (int c = 0; c < n; ++c) red[c][threadIdx.x] = v[c];
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st)
        for (int c = 0; c < n; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
      __syncthreads();
    }
    for (int c = 0; c < n; ++c) v[c] = red[c][0];
    __syncthreads();
  };
  if (origin == 2) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int a = threadIdx.x; a < numatm; a += blockDim.x) {
      const double w = agg_mass[a];
      if (w != 0.0) {
        v[0] += w;
        for (int c = 0; c < 3; ++c) v[1 + c] += w * pos[3 * (size_t)a + c];
      }
    }
    reduce(v, 4);
    if (threadIdx.x < 3) fit[threadIdx.x] = v[1 + threadIdx.x] / v[0];
    return;
  }
  double v[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int k = threadIdx.x; k < nh; k += blockDim.x) {
    const double w = ref_host[4 * k + 3];
    v[0] += w;
    for (int c = 0; c < 3; ++c) {
      v[1 + c] += w * pos[3 * (size_t)ref_atoms[k] + c];
      v[4 + c] += w * ref_host[4 * k + c];
    }
  }
  reduce(v, 7);
  double cf[3], cr[3];
  for (int c = 0; c < 3; ++c) {
    cf[c] = v[1 + c] / v[0];
    cr[c] = v[4 + c] / v[0];
  }
  double S9[9];
  for (int c = 0; c < 9; ++c) S9[c] = 0.0;
  for (int k = threadIdx.x; k < nh; k += blockDim.x) {
    const double w = ref_host[4 * k + 3];
    const int at = ref_atoms[k];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S9[3 * j + i] += (pos[3 * (size_t)at + i] - cf[i]) * (ref_host[4 * k + j] - cr[j]) * w;
  }
  reduce(S9, 9);
  if (threadIdx.x != 0) return;
  double S[3][3], q[4];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) S[j][i] = S9[3 * j + i];
  bestfit::rotation_quaternion(S, q);
  double* best = fit + 3 * (size_t)ns;  // refslt_bestfit
  for (int s = 0; s < ns; ++s) {
    const double b[3] = {ref_slt[4 * s], ref_slt[4 * s + 1], ref_slt[4 * s + 2]};
    bestfit::apply_fit(cf, cr, q, b, best + 3 * s);
  }
  // fit(refslt_natom, refslt_bestfit, bfcoord, refslt_weight, fit_sltcrd)
  double c1[3], c2[3], q2[4];
  bestfit::fit_transform(
      ns, [best](int s, int c) { return best[3 * s + c]; }, [bf](int s, int c) { return bf[3 * s + c]; },
      [ref_slt](int s) { return ref_slt[4 * s + 3]; }, c1, c2, q2);
  for (int s = 0; s < ns; ++s) bestfit::apply_fit(c1, c2, q2, bf + 3 * s, fit + 3 * s);
}

// getsolute's structure rejection (insertion.F90:438-467) over the whole library, one CTA:
// structure f passes when insstructure is 0, or when its best-fit RMSD from the reference
// solute (rmsd_bestfit, bestfit.F90:245-252: f fitted onto refslt_crd with refslt_weight,
// then rmsd_nofit) lies in [lw, up].  The passing structures are listed in file order in
// acc[0 .. na), na at acc[nconf].  FP64.
__global__ void __launch_bounds__(256) library_filter_kernel(const double* __restrict__ lib, int nconf, int ns,
                                                             int str, double lw, double up,
                                                             const double* __restrict__ rs, int* __restrict__ acc) {
  __shared__ int wtot[8];
  int base = 0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int f0 = 0; f0 < nconf; f0 += blockDim.x) {  // the same number of rounds in every thread
    const int f = f0 + (int)threadIdx.x;
    int pass = 0;
    if (f < nconf) {
      if (str == 0) {
        pass = 1;
      } else {
        const double* X = lib + (size_t)f * ns * 3;
        double cref[3], cx[3], q[4];
        bestfit::fit_transform(
            ns, [rs](int s, int c) { return rs[4 * s + c]; }, [X](int s, int c) { return X[3 * s + c]; },
            [rs](int s) { return rs[4 * s + 3]; }, cref, cx, q);
        double W = 0.0, disp = 0.0;
        for (int s = 0; s < ns; ++s) {
          double o[3];
          bestfit::apply_fit(cref, cx, q, X + 3 * s, o);
          double d2 = 0.0;
          for (int c = 0; c < 3; ++c) d2 += (o[c] - rs[4 * s + c]) * (o[c] - rs[4 * s + c]);
          W += rs[4 * s + 3];
          disp += rs[4 * s + 3] * d2;
        }
        const double d = sqrt(disp / W);
        pass = (lw <= d && d <= up) ? 1 : 0;
      }
    }
    // exclusive scan of pass over the block: the structure's place in the list
    const unsigned bal = __ballot_sync(0xffffffffu, pass);
    if (lane == 0) wtot[wid] = __popc(bal);
    __syncthreads();
    int off = base + __popc(bal & ((1u << lane) - 1u)), tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (w < wid) off += wtot[w];
      tot += wtot[w];
    }
    if (pass) acc[off] = f;
    base += tot;
    __syncthreads();  // wtot free for the next round
  }
  if (threadIdx.x == 0) acc[nconf] = base;
}

}  // namespace

cudaError_t launch_library_filter(Engine& e, int insstructure, double lwstr, double upstr) {
  library_filter_kernel<<<1, 256, 0, e.stream>>>(e.d_lib, e.lib_nconf, e.lib_ns, insstructure, lwstr, upstr,
                                                 e.d_ref_slt, e.d_lib_acc);
  e.count_launch();
  return cudaGetLastError();
}

cudaError_t launch_insert(Engine& e, int nplace, int ns, const ermod_insert_params& ip, const double* bf_d,
                          const double* mass_d, double* out, double* weight) {
  InsArgs A{};
  A.nplace = nplace;
  A.ns = ns;
  A.insposition = ip.insposition;
  A.insorient = ip.insorient;
  A.insorigin = ip.insorigin;
  A.lwreg = ip.lwreg;
  A.upreg = ip.upreg;
  A.k0 = (uint32_t)ip.seed;
  A.k1 = (uint32_t)(ip.seed >> 32);
  A.offset = ip.offset;
  for (int i = 0; i < 9; ++i) A.cell[i] = e.cell[i];
  A.bf = bf_d;
  A.mass = mass_d;
  A.out = out;
  A.weight = weight;
  A.status = e.d_status;
  if (e.lib_nconf > 0) {
    A.lib = e.d_lib;
    A.lib_wt = e.d_lib_wt;
    A.lib_acc = e.d_lib_acc;
    A.lib_nconf = e.lib_nconf;
    A.lib_nwt = e.lib_nwt;
    A.lib_na = e.lib_na;
  }
  if (ip.insorigin == 2 || ip.insorigin == 3) {
    insert_origin_kernel<<<1, 256, 0, e.stream>>>(e.d_sitepos, e.d_agg_mass, e.numatm, ip.insorigin, e.d_ref_atoms,
                                                  e.ref_nh, e.d_ref_host, e.d_ref_slt, ns, bf_d, e.d_ref_fit);
    e.count_launch();
    A.fit = e.d_ref_fit;
    A.rw = e.d_ref_slt;
  }
  const size_t smem = sizeof(double) * 4 * (size_t)ns;
  insert_kernel<<<(nplace + 127) / 128, 128, smem, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
