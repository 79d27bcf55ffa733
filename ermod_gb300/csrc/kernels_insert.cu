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
//   insorigin   0 COM to the origin, 1 as given
//   insposition 0 random in the cell (COM = cell U^3), 1 as given, 2 spherical shell
//               lwreg..upreg about the origin, 3/4 slab (generic / symmetric) in z,
//               5 random translation within upreg + 3 x solute size, 6 uniform /
//               Gaussian mixture with its WHAM weight (insertion.F90:274-316)
//   insorient   0 rotation about the COM by a unit quaternion from rejection sampling
//               of U[-1,1]^4 (applied as q v q*, bestfit.F90:75-100), 1 none
// The RMSD acceptance test of insposition 5 against a reference structure
// (check_solute_configuration) is not applied.
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
};

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
  for (int i = 0; i < 3 * A.ns; ++i) x[i] = sbf[i];
  double c[3];
  if (A.insorigin == 0) {  // set_solute_com(insml, 0)
    com_of(x, sm, A.ns, c);
    for (int s = 0; s < A.ns; ++s)
      for (int i = 0; i < 3; ++i) x[3 * s + i] -= c[i];
  }
  double weight = 1.0;
  double shift[3] = {0.0, 0.0, 0.0};
  bool ok = true;  // every rejection loop accepted
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
      if ((g & 1ull) == 0ull) {  // the reference starts with the uniform draw
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
  (void)ok;
  if (A.weight) A.weight[p] = weight;
}

}  // namespace

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
  const size_t smem = sizeof(double) * 4 * (size_t)ns;
  insert_kernel<<<(nplace + 127) / 128, 128, smem, e.stream>>>(A);
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
