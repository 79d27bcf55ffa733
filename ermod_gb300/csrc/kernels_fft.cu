// kernels_fft.cu -- the mixed path's PME solute potential: spectrum + 3-D C2R transform
// written for this path (replaces recpcal_prepare_solute's spread, R2C, engfac
// multiply and C2R, recpcal.F90:357-402, for a batch of placements).
//
//   pme_a   CTA per (k2, placement).  Generates the half-spectrum slab
//             S(k1, k3) = engfac(k1,k2,k3) sum_s q_s b1_s(k1) b2_s(k2) b3_s(k3)
//           (the exact R2C transform of the spread solute charges; b_{s,a} are the
//           1-D structure factors of the B-spline stencils), reduces the self energy
//           0.5 sum_k engfac |S|^2 (recpcal.F90:385-394; FP32 within a thread's tile,
//           float-float across tiles), and transforms the slab along k3 (inverse,
//           unnormalised) in shared memory.
//           Output T1[b][z][k2][k1] (complex FP32).
//   pme_b   CTA per (z, placement): the k2 transform of the (k2, k1) plane, then the
//           complex-to-real transform along k1, two rows per complex transform
//           (Z = X + iY); writes the real plane phi[b][z][y][x] with coalesced stores.
// Transforms are self-sorting Stockham passes (radices 2-16, composite radices done in
// registers), unnormalised, sign +1, exactly the conventions of fft_iface.F90.
#include <cooperative_groups.h>

#include "engine.cuh"

namespace ermod {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }  // a * i

// ---- in-register inverse DFTs: Y[q] = sum_r v[r] exp(+2 pi i r q / R) ----------------
template <int R>
struct Dft;

template <>
struct Dft<2> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};
template <>
struct Dft<3> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c = -0.5f, s = 0.86602540378443864676f;  // exp(2 pi i / 3)
    const float2 a = v[0], b = v[1], d = v[2];
    const float2 t = cadd(b, d), u = csub(b, d);
    v[0] = cadd(a, t);
    const float2 m = make_float2(a.x + c * t.x, a.y + c * t.y);
    const float2 n = make_float2(-s * u.y, s * u.x);  // i s (b - d)
    v[1] = cadd(m, n);
    v[2] = csub(m, n);
  }
};
template <>
struct Dft<4> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    const float2 c = cadd(v[1], v[3]), d = mul_i(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  }
};
template <>
struct Dft<5> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    const float2 a = v[0];
    const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const float2 u1 = csub(v[1], v[4]), u2 = csub(v[2], v[3]);
    v[0] = cadd(a, cadd(t1, t2));
    const float2 m1 = make_float2(a.x + c1 * t1.x + c2 * t2.x, a.y + c1 * t1.y + c2 * t2.y);
    const float2 m2 = make_float2(a.x + c2 * t1.x + c1 * t2.x, a.y + c2 * t1.y + c1 * t2.y);
    const float2 n1 = make_float2(s1 * u1.x + s2 * u2.x, s1 * u1.y + s2 * u2.y);  // (s1 u1 + s2 u2)
    const float2 n2 = make_float2(s2 * u1.x - s1 * u2.x, s2 * u1.y - s1 * u2.y);
    v[1] = cadd(m1, mul_i(n1));
    v[4] = csub(m1, mul_i(n1));
    v[2] = cadd(m2, mul_i(n2));
    v[3] = csub(m2, mul_i(n2));
  }
};

// compile-time cos/sin(pi x) for the in-register twiddles (Taylor series after reduction
// to [-1/2, 1/2]; |error| < 1e-16, folded to float constants)
constexpr double ct_pi = 3.14159265358979323846;
constexpr double ct_taylor_cos(double t) {  // cos(t), |t| <= pi/2
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term = -term * t * t / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}
constexpr double ct_taylor_sin(double t) {  // sin(t), |t| <= pi/2
  double term = t, sum = t;
  for (int k = 1; k < 16; ++k) {
    term = -term * t * t / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
constexpr double ct_cospi(double x) {  // cos(pi x)
  while (x > 1.0) x -= 2.0;
  while (x < -1.0) x += 2.0;
  if (x > 0.5) return -ct_taylor_cos(ct_pi * (1.0 - x));
  if (x < -0.5) return -ct_taylor_cos(ct_pi * (1.0 + x));
  return ct_taylor_cos(ct_pi * x);
}
constexpr double ct_sinpi(double x) {  // sin(pi x)
  while (x > 1.0) x -= 2.0;
  while (x < -1.0) x += 2.0;
  if (x > 0.5) return ct_taylor_sin(ct_pi * (1.0 - x));
  if (x < -0.5) return -ct_taylor_sin(ct_pi * (1.0 + x));
  return ct_taylor_sin(ct_pi * x);
}

// composite radix A*B in registers (Cooley-Tukey): B DFTs of size A on stride-B
// subsequences, twiddles exp(+2 pi i a b / R), then A DFTs of size B
template <int A, int B>
struct DftCT {
  static constexpr int R = A * B;
  static __device__ __forceinline__ void run(float2* v) {
    float2 t[R];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      float2 s[A];
#pragma unroll
      for (int a = 0; a < A; ++a) s[a] = v[a * B + b];
      Dft<A>::run(s);
#pragma unroll
      for (int a = 0; a < A; ++a) {
        if (a * b != 0) {
          const float cs = (float)ct_cospi(2.0 * (double)(a * b) / (double)R);
          const float sn = (float)ct_sinpi(2.0 * (double)(a * b) / (double)R);
          s[a] = cmul(s[a], make_float2(cs, sn));
        }
        t[a * B + b] = s[a];
      }
    }
    // t[a*B + b]: A-point results (index a) of subsequence b; now B-point DFTs over b
#pragma unroll
    for (int a = 0; a < A; ++a) {
      float2 s[B];
#pragma unroll
      for (int b = 0; b < B; ++b) s[b] = t[a * B + b];
      Dft<B>::run(s);
#pragma unroll
      for (int b = 0; b < B; ++b) v[b * A + a] = s[b];
    }
  }
};
template <>
struct Dft<6> : DftCT<2, 3> {};
template <>
struct Dft<8> : DftCT<2, 4> {};
template <>
struct Dft<9> : DftCT<3, 3> {};
template <>
struct Dft<10> : DftCT<2, 5> {};
template <>
struct Dft<12> : DftCT<4, 3> {};
template <>
struct Dft<15> : DftCT<3, 5> {};
template <>
struct Dft<16> : DftCT<4, 4> {};

// n / d for n < 2^16 by a multiply-high (m = ceil(2^32 / d)); d = 1 handled apart
struct FastDiv {
  unsigned d, m;
};
__host__ __device__ inline FastDiv make_fastdiv(unsigned d) {
  return FastDiv{d, d <= 1 ? 0u : (unsigned)((0x100000000ull + d - 1) / d)};
}
__device__ __forceinline__ int fdiv(int n, FastDiv f) { return f.d <= 1 ? n : (int)__umulhi((unsigned)n, f.m); }

// One Stockham pass of radix R over ncols transforms of length N (elements estride
// apart, transforms cstride apart), A -> B; consecutive threads take consecutive
// transforms, so the caller picks strides that keep shared-memory accesses conflict
// free.  tw[m] = exp(+2 pi i m / N).
template <int R>
__device__ __forceinline__ void stockham_pass(const float2* __restrict__ A, float2* __restrict__ B, int N, int Ns,
                                              FastDiv fNs, int ncols, FastDiv fcols, int estride, int cstride,
                                              int oestride, int ocstride, const float2* __restrict__ tw) {
  const int NR = N / R;
  const int total = ncols * NR;
  const int step = N / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int j = fdiv(t, fcols);
    const int col = t - j * ncols;
    const int jq = fdiv(j, fNs);
    const int k = j - jq * Ns;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = A[col * cstride + (j + r * NR) * estride];
    if (k > 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * k * step]);  // r k step < N
    }
    Dft<R>::run(v);
    const int idxD = jq * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) B[(size_t)col * ocstride + (size_t)(idxD + r * Ns) * oestride] = v[r];
  }
}

__device__ __forceinline__ void run_pass(int R, const float2* A, float2* B, int N, int Ns, FastDiv fNs, int ncols,
                                         FastDiv fcols, int estride, int cstride, int oestride, int ocstride,
                                         const float2* tw) {
#define ERMOD_PASS(RR) \
  case RR: stockham_pass<RR>(A, B, N, Ns, fNs, ncols, fcols, estride, cstride, oestride, ocstride, tw); break;
  switch (R) {
    ERMOD_PASS(2)
    ERMOD_PASS(3)
    ERMOD_PASS(4)
    ERMOD_PASS(5)
    ERMOD_PASS(6)
    ERMOD_PASS(8)
    ERMOD_PASS(9)
    ERMOD_PASS(10)
    ERMOD_PASS(12)
    ERMOD_PASS(15)
    ERMOD_PASS(16)
    default: break;
  }
#undef ERMOD_PASS
}

}  // namespace

// radix plan: at most kMaxPasses radices from {16,15,12,10,9,8,6,5,4,3,2}, fewest passes
constexpr int kMaxPasses = 6;
struct FftPlan {
  int n, npass, r[kMaxPasses], ns[kMaxPasses];
  FastDiv fns[kMaxPasses];
};

bool make_fft_plan(int n, FftPlan& p) {
  static const int cand[] = {16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};
  p.n = n;
  p.npass = 0;
  // prefer two balanced passes when possible
  for (int a : cand)
    if (n % a == 0) {
      const int b = n / a;
      for (int c : cand)
        if (c == b) {
          p.npass = 2;
          p.r[0] = a;
          p.r[1] = b;
          return true;
        }
    }
  for (int a : cand)  // a single pass
    if (a == n) {
      p.npass = 1;
      p.r[0] = a;
      return true;
    }
  int m = n;
  while (m > 1 && p.npass < kMaxPasses) {
    bool found = false;
    for (int a : cand)
      if (m % a == 0) {
        p.r[p.npass++] = a;
        m /= a;
        found = true;
        break;
      }
    if (!found) return false;
  }
  if (n == 1) {
    p.npass = 0;
    return true;
  }
  return m == 1;
}

static bool finish_plan(FftPlan& p) {
  int ns = 1;
  for (int i = 0; i < p.npass; ++i) {
    p.ns[i] = ns;
    p.fns[i] = make_fastdiv((unsigned)ns);
    ns *= p.r[i];
  }
  return ns == p.n;
}

static bool plan(int n, FftPlan& p) { return make_fft_plan(n, p) && finish_plan(p); }

namespace {

// inverse transform of ncols columns; data starts in A, ends in the returned buffer
__device__ __forceinline__ float2* fft_cols(float2* A, float2* B, const FftPlan& pl, int ncols, FastDiv fcols,
                                            int estride, int cstride, const float2* tw) {
  for (int p = 0; p < pl.npass; ++p) {
    __syncthreads();
    run_pass(pl.r[p], A, B, pl.n, pl.ns[p], pl.fns[p], ncols, fcols, estride, cstride, estride, cstride, tw);
    float2* t = A;
    A = B;
    B = t;
  }
  __syncthreads();
  return A;
}

// the same with the first pass reading `in` (element/column strides ies/ics, e.g. a
// plane in global memory) and the last pass writing `out` (strides oes/ocs); the
// intermediate passes ping-pong between the shared buffers A and B (npass >= 2)
__device__ __forceinline__ void fft_cols_io(const float2* in, int ies, int ics, float2* A, float2* B,
                                            const FftPlan& pl, int ncols, FastDiv fcols, int estride, int cstride,
                                            float2* out, int oes, int ocs, const float2* tw) {
  const float2* src = in;
  int se = ies, sc = ics;
  for (int p = 0; p < pl.npass; ++p) {
    const bool lastp = (p == pl.npass - 1);
    float2* dst = lastp ? out : ((p & 1) ? B : A);
    __syncthreads();
    run_pass(pl.r[p], src, dst, pl.n, pl.ns[p], pl.fns[p], ncols, fcols, se, sc, lastp ? oes : estride,
             lastp ? ocs : cstride, tw);
    src = dst;
    se = estride;
    sc = cstride;
  }
}

// ---- compile-time plans for cubic grids of a few common sizes ----------------------
// The same two Stockham passes as fft_cols_io, with the transform length, radices,
// column count, strides and thread count known to the compiler, so that the index
// arithmetic (the ALU share of the transforms) folds into constants.
constexpr int kPmeAThreads = 512;  // pme_a's largest CTA

constexpr bool radix_ok(int r) {
  return r == 16 || r == 15 || r == 12 || r == 10 || r == 9 || r == 8 || r == 6 || r == 5 || r == 4 || r == 3 ||
         r == 2;
}
constexpr int first_radix(int n) {  // make_fft_plan's two-pass choice (first radix from the top)
  return (n % 16 == 0 && radix_ok(n / 16)) ? 16
       : (n % 15 == 0 && radix_ok(n / 15)) ? 15
       : (n % 12 == 0 && radix_ok(n / 12)) ? 12
       : (n % 10 == 0 && radix_ok(n / 10)) ? 10
       : (n % 9 == 0 && radix_ok(n / 9))   ? 9
       : (n % 8 == 0 && radix_ok(n / 8))   ? 8
       : (n % 6 == 0 && radix_ok(n / 6))   ? 6
                                           : 0;
}

template <int R, int N, int NS, int NCOLS, int IES, int ICS, int OES, int OCS, int NT>
__device__ __forceinline__ void stockham_pass_t(const float2* __restrict__ A, float2* __restrict__ B,
                                                const float2* __restrict__ tw) {
  constexpr int NR = N / R, TOTAL = NCOLS * NR, STEP = N / (NS * R);
  for (int t = threadIdx.x; t < TOTAL; t += NT) {
    const int j = t / NCOLS;
    const int col = t - j * NCOLS;
    const int jq = j / NS;
    const int k = j - jq * NS;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = A[col * ICS + (j + r * NR) * IES];
    if (NS > 1 && k > 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * k * STEP]);
    }
    Dft<R>::run(v);
    const int idxD = jq * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) B[(size_t)col * OCS + (size_t)(idxD + r * NS) * OES] = v[r];
  }
}

// two passes: in (IES, ICS) -> mid (ES, CS) -> out (OES, OCS); each pass starts with a barrier
template <int N, int NCOLS, int IES, int ICS, int ES, int CS, int OES, int OCS, int NT>
__device__ __forceinline__ void fft2_t(const float2* in, float2* mid, float2* out, const float2* tw) {
  constexpr int R0 = first_radix(N), R1 = N / R0;
  static_assert(R0 > 0 && radix_ok(R1), "no two-pass plan");
  __syncthreads();
  stockham_pass_t<R0, N, 1, NCOLS, IES, ICS, ES, CS, NT>(in, mid, tw);
  __syncthreads();
  stockham_pass_t<R1, N, R0, NCOLS, ES, CS, OES, OCS, NT>(mid, out, tw);
}

// lengths without a two-pass plan: make_fft_plan's greedy radices (largest first)
constexpr int greedy_radix(int n) {
  return n % 16 == 0 ? 16 : n % 15 == 0 ? 15 : n % 12 == 0 ? 12 : n % 10 == 0 ? 10 : n % 9 == 0 ? 9
       : n % 8 == 0 ? 8 : n % 6 == 0 ? 6 : n % 5 == 0 ? 5 : n % 4 == 0 ? 4 : n % 3 == 0 ? 3 : n % 2 == 0 ? 2 : 0;
}
constexpr bool two_pass(int n) { return first_radix(n) > 0; }

// three passes: in -> mid -> mid2 -> out (mid2 may be the buffer `in` when that is shared
// memory the first pass has consumed)
template <int N, int NCOLS, int IES, int ICS, int ES, int CS, int OES, int OCS, int NT>
__device__ __forceinline__ void fft3_t(const float2* in, float2* mid, float2* mid2, float2* out, const float2* tw) {
  constexpr int R0 = greedy_radix(N), R1 = greedy_radix(N / R0), R2 = N / (R0 * R1);
  static_assert(R0 > 0 && R1 > 0 && radix_ok(R2) && R0 * R1 * R2 == N, "no three-pass plan");
  __syncthreads();
  stockham_pass_t<R0, N, 1, NCOLS, IES, ICS, ES, CS, NT>(in, mid, tw);
  __syncthreads();
  stockham_pass_t<R1, N, R0, NCOLS, ES, CS, ES, CS, NT>(mid, mid2, tw);
  __syncthreads();
  stockham_pass_t<R2, N, R0 * R1, NCOLS, ES, CS, OES, OCS, NT>(mid2, out, tw);
}

constexpr int kSites = 32;  // solute sites staged per chunk
constexpr int kR1 = 4, kR3 = 3;  // generation tile: kR3 k3 values x kR1 k1 values per thread
static_assert(kR1 == 4, "pme_a reads a tile row's engfac values as one float4");

// Large grids in pme_a: a work buffer as large as the slab would leave room for one CTA
// per SM, so the k3 transform runs over two halves of the columns through a work buffer
// of half the slab's columns (and the site staging takes smaller chunks to fit in it).
constexpr int pme_a_hp(int KC) { return ((KC / 2 + 1 + kR1 - 1) / kR1) * kR1; }
// CTA size of the compile-time PME kernels: one thread per generation tile (kR3 x kR1
// points), rounded up to whole warps and capped at 512, and as many CTAs per SM as its
// registers allow at 64 per thread.  Small grids have few transform columns and tiles, so
// their CTAs are small and many share an SM; at 96^3, 416 threads for the 13 x 32 tiles
// (measured +0.8% on the 33,000-water workload against 512, every transform pass but the
// last in one round).
constexpr int pme_tiles(int KC) { return (pme_a_hp(KC) / kR1) * ((KC + kR3 - 1) / kR3); }
constexpr int pme_threads(int KC) {
  return KC == 0 ? 512 : (((pme_tiles(KC) + 31) / 32) * 32 > 512 ? 512 : ((pme_tiles(KC) + 31) / 32) * 32);
}
constexpr int pme_min_blocks(int KC) {
  return 65536 / (pme_threads(KC) * 64) > 16 ? 16 : 65536 / (pme_threads(KC) * 64);
}
static_assert(pme_threads(96) == 416 && pme_threads(80) == 320 && pme_threads(128) == 512 && pme_threads(32) == 64,
              "CTA sizes");

constexpr bool pme_a_halves(int KC) {  // cubic grids with compile-time sizes (KC > 0)
  return KC > 0 && two_pass(KC) && sizeof(float2) * ((size_t)2 * KC * pme_a_hp(KC) + KC) > 110 * 1024;
}
constexpr int pme_a_work_cols(int KC) { return pme_a_halves(KC) ? (KC / 2 + 2) / 2 : pme_a_hp(KC); }

struct PmeArgs {
  const float2* bvec;   // [nb][S][3][Kmax]
  const float* u_qf;    // [nb][S]
  const int* u_nsite;
  const float* engfac;  // [K3][K2][Hp], zeros beyond H
  const float2* twiddle;  // per axis, exp(-2 pi i m / K): conjugated here for the inverse
  float2* t1;           // [nb][K3][K2][H]
  float* phi;           // [nb][K3][K2][K1]
  double* self_part;    // [nb][K2]
  int nb, K1, K2, K3, H, Hp, K1p, Kmax;
  int chunk;  // solute sites staged per generation chunk (fits the k3 work buffer)
  int halo, XP, YP, ZP;  // padded periodic potential grid (see pme_b)
  FftPlan p1, p2, p3;
  FastDiv fH, fK1, fHp4, fnpair, fKX;
};

// KC > 0: a K^3 grid with K = KC and compile-time transforms; KC = 0: any grid
template <int KC>
__global__ void __launch_bounds__(pme_threads(KC), pme_min_blocks(KC)) pme_a_kernel(PmeArgs A) {
  extern __shared__ float2 sm[];
  const int k2 = blockIdx.x, b = blockIdx.y;
  // compile-time sizes when specialised (the runtime values are then equal)
  const int K3 = KC ? KC : A.K3, H = KC ? KC / 2 + 1 : A.H;
  const int Hp = KC ? ((KC / 2 + 1 + kR1 - 1) / kR1) * kR1 : A.Hp;
  float2* slab = sm;                          // [K3][Hp]
  float2* work = sm + (size_t)K3 * Hp;        // [K3][Hp or half of it]; site staging during generation
  float2* tw3 = work + (size_t)K3 * (KC ? pme_a_work_cols(KC) : Hp);  // [K3]
  const int ns = A.u_nsite[b];
  for (int i = threadIdx.x; i < K3; i += blockDim.x) {
    const float2 t = A.twiddle[A.K1 + A.K2 + i];
    tw3[i] = make_float2(t.x, -t.y);
  }
  const float2* bv = A.bvec + (size_t)b * kMaxSoluteSites * 3 * A.Kmax;
  const int TX = Hp / kR1, TY = (K3 + kR3 - 1) / kR3;
  const bool even = (A.K1 % 2) == 0;
  ff self{0.f, 0.f};
  // ---- generation: slab(k3, k1) = sum_s [q_s b2_s(k2) b3_s(k3)] b1_s(k1), then (last
  // chunk) the engfac multiply and the self energy sum 0.5 sum_k engfac |S|^2 ----
  float2* sd = work;                         // [chunk][K3]
  // [chunk][kR1][TX]: b1(k1 = kR1 tx + i) at [i][tx], so that the lanes of a warp (consecutive
  // tx) read consecutive words
  float2* sb = work + (size_t)A.chunk * K3;
  for (int s0 = 0; s0 < ns; s0 += A.chunk) {
    const int nsc = min(A.chunk, ns - s0);
    const bool last = s0 + A.chunk >= ns;
    __syncthreads();
    // staging: each thread first issues the loads of its entries of both tables (and the
    // first nsc threads those of q b2(k2) per site), then forms and stores them, so that
    // one L2 round trip covers its share (issued one entry at a time, the round trips made
    // the staging about a third of the CTA's time)
    constexpr int kStage = 2;
    const int nd = nsc * K3, n1 = nsc * Hp;
    __shared__ float2 sqb2[kSites];  // q_s b2_s(k2)
    for (int r0 = 0; r0 < max(nd, n1); r0 += kStage * blockDim.x) {
      const int base = r0 + (int)threadIdx.x;
      float2 b3[kStage], b1[kStage];
#pragma unroll
      for (int i = 0; i < kStage; ++i) {
        const int t = base + i * blockDim.x;
        if (t < nd) {
          const int sl = t / K3, k3 = t - sl * K3;
          b3[i] = bv[((size_t)(s0 + sl) * 3 + 2) * A.Kmax + k3];
        }
        if (t < n1) {
          const int sl = t / Hp, k1 = t - sl * Hp;
          b1[i] = (k1 < H) ? bv[((size_t)(s0 + sl) * 3 + 0) * A.Kmax + k1] : make_float2(0.f, 0.f);
        }
      }
      if (r0 == 0 && threadIdx.x < (unsigned)nsc) {
        const size_t us = (size_t)(s0 + threadIdx.x);
        const float q = A.u_qf[(size_t)b * kMaxSoluteSites + us];
        const float2 b2 = bv[(us * 3 + 1) * A.Kmax + k2];
        sqb2[threadIdx.x] = make_float2(q * b2.x, q * b2.y);
      }
      __syncthreads();  // sqb2 staged (the loop runs the same number of rounds in every thread)
#pragma unroll
      for (int i = 0; i < kStage; ++i) {
        const int t = base + i * blockDim.x;
        if (t < nd) {
          const int sl = t / K3, k3 = t - sl * K3;
          sd[sl * K3 + k3] = cmul(sqb2[sl], b3[i]);
        }
        if (t < n1) {
          const int sl = t / Hp, k1 = t - sl * Hp;
          sb[sl * Hp + (k1 % kR1) * TX + k1 / kR1] = b1[i];
        }
      }
    }
    __syncthreads();
    for (int mt = threadIdx.x; mt < TX * TY; mt += blockDim.x) {
      const int ty = KC ? mt / TX : fdiv(mt, A.fHp4), tx = mt - ty * TX;
      const int k1a = tx * kR1, k3a = ty * kR3;
      float2 acc[kR3][kR1];
#pragma unroll
      for (int j = 0; j < kR3; ++j)
#pragma unroll
        for (int i = 0; i < kR1; ++i) acc[j][i] = make_float2(0.f, 0.f);
      for (int sl = 0; sl < nsc; ++sl) {
        float2 d[kR3], e[kR1];
#pragma unroll
        for (int j = 0; j < kR3; ++j) d[j] = (k3a + j < K3) ? sd[sl * K3 + k3a + j] : make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < kR1; ++i) e[i] = sb[sl * Hp + i * TX + tx];
#pragma unroll
        for (int j = 0; j < kR3; ++j)
#pragma unroll
          for (int i = 0; i < kR1; ++i) {
            acc[j][i].x = fmaf(d[j].x, e[i].x, fmaf(-d[j].y, e[i].y, acc[j][i].x));
            acc[j][i].y = fmaf(d[j].x, e[i].y, fmaf(d[j].y, e[i].x, acc[j][i].y));
          }
      }
      float tile_self = 0.f;  // the tile's self-energy terms (all >= 0), summed in FP32
#pragma unroll
      for (int j = 0; j < kR3; ++j) {
        const int k3 = k3a + j;
        if (k3 >= K3) continue;
        float4* dst = reinterpret_cast<float4*>(slab + (size_t)k3 * Hp + k1a);
        if (s0 != 0) {
          const float4 o0 = dst[0], o1 = dst[1];
          acc[j][0] = cadd(acc[j][0], make_float2(o0.x, o0.y));
          acc[j][1] = cadd(acc[j][1], make_float2(o0.z, o0.w));
          acc[j][2] = cadd(acc[j][2], make_float2(o1.x, o1.y));
          acc[j][3] = cadd(acc[j][3], make_float2(o1.z, o1.w));
        }
        if (last) {  // FP32 engfac rows are Hp points long, zeros beyond H
          const float4 f4 = __ldg(reinterpret_cast<const float4*>(A.engfac + ((size_t)k3 * A.K2 + k2) * Hp + k1a));
          const float fv[kR1] = {f4.x, f4.y, f4.z, f4.w};
#pragma unroll
          for (int i = 0; i < kR1; ++i) {
            const int k1 = k1a + i;
            const float f = fv[i];
            const float2 q = acc[j][i];
            const float wgt = (k1 == 0 || (even && k1 == H - 1)) ? 0.5f : 1.f;
            tile_self += wgt * f * (q.x * q.x + q.y * q.y);
            acc[j][i] = make_float2(f * q.x, f * q.y);
          }
        }
        dst[0] = make_float4(acc[j][0].x, acc[j][0].y, acc[j][1].x, acc[j][1].y);
        dst[1] = make_float4(acc[j][2].x, acc[j][2].y, acc[j][3].x, acc[j][3].y);
      }
      if (last) self = ff_add(self, tile_self);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    ff o{__shfl_down_sync(0xffffffffu, self.hi, off), __shfl_down_sync(0xffffffffu, self.lo, off)};
    self = ff_add2(self, o);
  }
  // the warps' float-float sums, combined in FP32 by one thread: an FP64 instruction costs
  // GB300 as much as 64 FP32 ones, so the CTA converts to FP64 once
  __shared__ float2 wsum[kPmeAThreads / 32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = make_float2(self.hi, self.lo);
  // ---- inverse transform along k3 (columns k1, element stride Hp); the last pass
  // writes T1[b][z][k2][k1] ----
  float2* out = A.t1 + (size_t)b * K3 * A.K2 * H + (size_t)k2 * H;
  if constexpr (KC > 0) {
    constexpr int HC = KC / 2 + 1, HPC = ((HC + kR1 - 1) / kR1) * kR1;
    if constexpr (pme_a_halves(KC)) {  // columns [0, HA), then [HA, HC), through a half buffer
      constexpr int HA = (HC + 1) / 2, HB = HC - HA;
      fft2_t<KC, HA, HPC, 1, HA, 1, KC * HC, 1, pme_threads(KC)>(slab, work, out, tw3);
      fft2_t<KC, HB, HPC, 1, HB, 1, KC * HC, 1, pme_threads(KC)>(slab + HA, work, out + HA, tw3);
    } else if constexpr (two_pass(KC))
      fft2_t<KC, HC, HPC, 1, HPC, 1, KC * HC, 1, pme_threads(KC)>(slab, work, out, tw3);
    else
      fft3_t<KC, HC, HPC, 1, HPC, 1, KC * HC, 1, pme_threads(KC)>(slab, work, slab, out, tw3);
  } else {
    fft_cols_io(slab, Hp, 1, work, slab, A.p3, H, A.fH, Hp, 1, out, A.K2 * H, 1, tw3);
  }
  if (threadIdx.x == 0) {
    ff t{0.f, 0.f};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = ff_add2(t, ff{wsum[w].x, wsum[w].y});
    A.self_part[(size_t)b * A.K2 + k2] = ff_to_double(t);
  }
}

// The two passes around the row-pair layout of pme_b_planes_fused.  pass_to_pairs: the
// second k2 pass (radix R1 = K / R0, NS = R0, columns k1) storing element (k2, k1) at
// [k2 / 2][k1][k2 % 2], pairs 2H apart.  NC columns starting at column c0 of the plane,
// read from a buffer whose rows (fixed k2) are IS elements long.
template <int KC, int NC = KC / 2 + 1, int IS = KC / 2 + 1>
__device__ __forceinline__ void pass_to_pairs(const float2* __restrict__ A, float2* __restrict__ B,
                                              const float2* __restrict__ tw, int c0 = 0) {
  constexpr int HC = KC / 2 + 1, R0 = first_radix(KC), R = KC / R0, NR = KC / R, SP = 2 * HC;
  if constexpr (R0 % 2 == 0) {
    // a thread transforms the adjacent columns j, j + 1 (j even): their outputs e, e + 1
    // are the two rows of one pair, stored with one 16-byte, conflict-free store
    for (int t = threadIdx.x; t < NC * (NR / 2); t += pme_threads(KC)) {
      const int jp = t / NC;
      const int col = t - jp * NC;
      const int j = 2 * jp;
      float2 v0[R], v1[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        v0[r] = A[col + (j + r * NR) * IS];
        v1[r] = A[col + (j + 1 + r * NR) * IS];
      }
#pragma unroll
      for (int r = 1; r < R; ++r) {
        if (j > 0) v0[r] = cmul(v0[r], tw[r * j]);
        v1[r] = cmul(v1[r], tw[r * (j + 1)]);
      }
      Dft<R>::run(v0);
      Dft<R>::run(v1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int e = j + r * R0;  // even
        *reinterpret_cast<float4*>(B + (e >> 1) * SP + 2 * (c0 + col)) =
            make_float4(v0[r].x, v0[r].y, v1[r].x, v1[r].y);
      }
    }
  } else {
    for (int t = threadIdx.x; t < NC * NR; t += pme_threads(KC)) {
      const int j = t / NC;  // < NR = R0 = NS, so the pass's k is j
      const int col = t - j * NC;
      float2 v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = A[col + (j + r * NR) * IS];
      if (j > 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * j]);
      }
      Dft<R>::run(v);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int e = j + r * R0;
        B[(e >> 1) * SP + 2 * (c0 + col) + (e & 1)] = v[r];
      }
    }
  }
}

// pass_from_pairs: the first row pass (radix R0, no twiddles, K / 2 row pairs) packing
// Z_p[k] = X_{2p}[k] + i X_{2p+1}[k] while it loads, Hermitian-completed in k1 (the upper
// half of k1 is the conjugate of the stored half); rows K | 1 apart in B.  NPH pairs
// starting at pair p0 of A, written from row 0 of B.
template <int KC, int NPH = KC / 2>
__device__ __forceinline__ void pass_from_pairs(const float2* __restrict__ A, float2* __restrict__ B, int p0 = 0) {
  constexpr int HC = KC / 2 + 1, R = first_radix(KC), NR = KC / R, SP = 2 * HC, RS = KC | 1;
  for (int t = threadIdx.x; t < NPH * NR; t += pme_threads(KC)) {
    const int j = t / NPH;
    const int p = t - j * NPH;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = j + r * NR;
      const int kk = k < HC ? k : KC - k;
      const float4 q = *reinterpret_cast<const float4*>(A + (p0 + p) * SP + 2 * kk);
      float2 x0 = make_float2(q.x, q.y), x1 = make_float2(q.z, q.w);
      if (k >= HC) {
        x0.y = -x0.y;
        x1.y = -x1.y;
      }
      if (k == 0 || k == KC / 2) {  // self-conjugate points
        x0.y = 0.f;
        x1.y = 0.f;
      }
      v[r] = make_float2(x0.x - x1.y, x0.y + x1.x);
    }
    Dft<R>::run(v);
#pragma unroll
    for (int r = 0; r < R; ++r) B[p * RS + j * R + r] = v[r];
  }
}

// pme_b_planes for cubic two-pass grids with K a multiple of 4 (H odd): the k2 transform
// leaves rows 2p and 2p + 1 interleaved point by point ([p][k1][2], pairs 2H apart), and
// the first pass of the row transforms packs the pairs while it loads them (one 16-byte
// load per point, conflict free as H is odd), so there is no separate packing pass.
template <int KC>
__device__ __forceinline__ float2* pme_b_planes_fused(const float2* in, float2* s0, float2* s1, const float2* tw) {
  constexpr int HC = KC / 2 + 1, R0 = first_radix(KC), R1 = KC / R0, RS = KC | 1;
  __syncthreads();
  stockham_pass_t<R0, KC, 1, HC, HC, 1, HC, 1, pme_threads(KC)>(in, s0, tw);
  __syncthreads();
  pass_to_pairs<KC>(s0, s1, tw);
  __syncthreads();
  pass_from_pairs<KC>(s1, s0);
  __syncthreads();
  stockham_pass_t<R1, KC, R0, KC / 2, 1, RS, 1, RS, pme_threads(KC)>(s0, s1, tw);
  __syncthreads();
  return s1;
}

// Large grids: two full plane buffers would leave room for one CTA per SM, so the plane
// stays in one full buffer A and every transform runs in two halves through a buffer W of
// half its size -- the k2 transforms over the left and then the right half of the columns
// (first pass plane -> W, second W -> A in the pair layout), the row transforms over the
// first and then the second half of the row pairs (first pass A -> W, second W -> A as
// rows K | 1 apart: a half's rows end below the pairs the other half still reads).
constexpr bool pme_b_halves(int KC) {  // cubic grids with compile-time sizes (KC > 0)
  return KC > 0 && two_pass(KC) && KC % 4 == 0 &&
         sizeof(float2) * (2 * (size_t)(KC / 2 + 1) * KC + KC) > 110 * 1024;
}
constexpr size_t pme_b_half_w(int KC) {  // W in float2: the wider half of either phase
  return (size_t)KC * ((KC / 2 + 2) / 2) > (size_t)((KC / 2 + 1) / 2) * (KC | 1)
             ? (size_t)KC * ((KC / 2 + 2) / 2)
             : (size_t)((KC / 2 + 1) / 2) * (KC | 1);
}

template <int KC>
__device__ __forceinline__ float2* pme_b_planes_halves(const float2* in, float2* A, float2* W,
                                                       const float2* tw) {
  constexpr int HC = KC / 2 + 1, R0 = first_radix(KC), R1 = KC / R0, RS = KC | 1, NP = KC / 2;
  constexpr int HA = (HC + 1) / 2, HB = HC - HA;  // column halves
  constexpr int PA = (NP + 1) / 2, PB = NP - PA;  // row-pair halves
  __syncthreads();
  stockham_pass_t<R0, KC, 1, HA, HC, 1, HA, 1, pme_threads(KC)>(in, W, tw);
  __syncthreads();
  pass_to_pairs<KC, HA, HA>(W, A, tw, 0);
  __syncthreads();
  stockham_pass_t<R0, KC, 1, HB, HC, 1, HB, 1, pme_threads(KC)>(in + HA, W, tw);
  __syncthreads();
  pass_to_pairs<KC, HB, HB>(W, A, tw, HA);
  __syncthreads();
  pass_from_pairs<KC, PA>(A, W, 0);
  __syncthreads();
  stockham_pass_t<R1, KC, R0, PA, 1, RS, 1, RS, pme_threads(KC)>(W, A, tw);
  __syncthreads();
  pass_from_pairs<KC, PB>(A, W, PA);
  __syncthreads();
  stockham_pass_t<R1, KC, R0, PB, 1, RS, 1, RS, pme_threads(KC)>(W, A + (size_t)PA * RS, tw);
  __syncthreads();
  return A;
}

// the plane's k2 transforms, a separate pass that packs row pairs (Hermitian-completed in
// k1) into rows K1p apart, and the row transforms; returns the buffer holding the result
template <int KC>
__device__ __forceinline__ float2* pme_b_planes(const PmeArgs& A, const float2* in, float2* s0, float2* s1,
                                                const float2* tw1, const float2* tw2) {
  const int K1 = KC ? KC : A.K1, K2 = KC ? KC : A.K2;
  const int H = KC ? KC / 2 + 1 : A.H, K1p = KC ? (KC | 1) : A.K1p;
  const int npair = (K2 + 1) / 2;
  // k2 transform: columns k1 (stride 1), elements along k2 (stride H); the first pass
  // reads the plane from global memory
  const int np2 = A.p2.npass;
  float2* r = (np2 == 1) ? s0 : ((((np2 - 2) & 1) ? s0 : s1));  // not the last pass's source
  if constexpr (KC > 0) {
    constexpr int HC = KC / 2 + 1;
    if constexpr (two_pass(KC))
      fft2_t<KC, HC, HC, 1, HC, 1, HC, 1, pme_threads(KC)>(in, s0, r, tw2);
    else  // r is s0 for three passes (the runtime plan's count)
      fft3_t<KC, HC, HC, 1, HC, 1, HC, 1, pme_threads(KC)>(in, s0, s1, r, tw2);
  } else {
    fft_cols_io(in, H, 1, s0, s1, A.p2, H, A.fH, H, 1, r, H, 1, tw2);
  }
  __syncthreads();
  float2* w = (r == s0) ? s1 : s0;
  // pack row pairs: Z_p[k] = X_{2p}[k] + i X_{2p+1}[k], Hermitian-completed in k1;
  // rows padded to K1p (odd) so the row transforms are bank-conflict free
  // one warp per row pair, lanes along k1 (no division); the upper half of k1 is the
  // conjugate of the stored half
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  if constexpr (KC > 0) {
    // the lane's columns k = lane + 32 i, their mirrored source and flags, set up once
    constexpr int NK = (KC + 31) / 32, HC = KC / 2 + 1;
    int kk[NK];
    unsigned conj = 0u, real = 0u;
#pragma unroll
    for (int i = 0; i < NK; ++i) {
      const int k = lane + 32 * i;
      kk[i] = k < HC ? k : KC - k;
      if (k >= HC) conj |= 1u << i;
      if (k == 0 || ((KC % 2 == 0) && k == KC / 2)) real |= 1u << i;  // self-conjugate points
    }
    for (int pp = warp; pp < npair; pp += nwarp) {
      const float2* r0 = r + (size_t)(2 * pp) * HC;
      const float2* r1 = r0 + HC;
      const bool has1 = 2 * pp + 1 < KC;
      float2* wrow = w + (size_t)pp * (KC | 1) + lane;
#pragma unroll
      for (int i = 0; i < NK; ++i) {
        if (KC % 32 != 0 && lane + 32 * i >= KC) break;
        float2 x0 = r0[kk[i]];
        float2 x1 = has1 ? r1[kk[i]] : make_float2(0.f, 0.f);
        if (conj & (1u << i)) {
          x0.y = -x0.y;
          x1.y = -x1.y;
        }
        if (real & (1u << i)) {
          x0.y = 0.f;
          x1.y = 0.f;
        }
        wrow[32 * i] = make_float2(x0.x - x1.y, x0.y + x1.x);
      }
    }
  } else {
    for (int pp = warp; pp < npair; pp += nwarp) {
      const float2* r0 = r + (size_t)(2 * pp) * H;
      const float2* r1 = r0 + H;
      const bool has1 = 2 * pp + 1 < K2;
      float2* wrow = w + (size_t)pp * K1p;
      for (int k = lane; k < K1; k += 32) {
        const bool lo = k < H;
        const int kk = lo ? k : K1 - k;
        float2 x0 = r0[kk];
        float2 x1 = has1 ? r1[kk] : make_float2(0.f, 0.f);
        if (!lo) {
          x0.y = -x0.y;
          x1.y = -x1.y;
        }
        if (k == 0 || ((K1 % 2 == 0) && k == K1 / 2)) {  // self-conjugate points
          x0.y = 0.f;
          x1.y = 0.f;
        }
        wrow[k] = make_float2(x0.x - x1.y, x0.y + x1.x);
      }
    }
  }
  float2* res;
  if constexpr (KC > 0) {  // ping-pong between w and r: w -> r -> w (-> r)
    // (KC + 1) / 2 row pairs (the last one a single row when KC is odd), rows KC | 1 apart
    if constexpr (two_pass(KC)) {
      fft2_t<KC, (KC + 1) / 2, 1, (KC | 1), 1, (KC | 1), 1, (KC | 1), pme_threads(KC)>(w, r, w, tw1);
      res = w;
    } else {
      fft3_t<KC, (KC + 1) / 2, 1, (KC | 1), 1, (KC | 1), 1, (KC | 1), pme_threads(KC)>(w, r, w, r, tw1);
      res = r;
    }
    __syncthreads();
  } else {
    res = fft_cols(w, r, A.p1, npair, A.fnpair, 1, K1p, tw1);
  }
  return res;
}

// CTA per (z, placement): the k2 transform of the (k2, k1) plane, then the
// complex-to-real transform along k1, two rows per complex transform; writes the real
// plane into the placement's lane of the interleaved potential grid.
// Compile-time sizes (KC > 0): the four CTAs of an interleaved group (the same plane of
// four placements) form a thread-block cluster.  Once their planes are done, each CTA
// reads a quarter of the rows of all four planes through distributed shared memory and
// writes them as whole float4 points (16-byte stores, full 32-byte sectors), instead of
// every CTA storing 4 bytes at a 16-byte stride (a quarter-used sector per store).
template <int KC>
__global__ void __launch_bounds__(pme_threads(KC), pme_min_blocks(KC)) pme_b_kernel(PmeArgs A) {
  extern __shared__ __align__(16) float2 sm[];  // 16-byte loads of row pairs
  // grid (4, K3, ceil(nb / 4)): the four placements that share an interleaved potential
  // grid run side by side
  const int z = blockIdx.y, b = 4 * blockIdx.z + blockIdx.x;
  const bool live = b < A.nb;  // the last group may hold fewer than four placements
  if constexpr (KC == 0) {
    if (!live) return;
  }
  const int K1 = KC ? KC : A.K1, K2 = KC ? KC : A.K2, K3 = KC ? KC : A.K3;
  const int H = KC ? KC / 2 + 1 : A.H, K1p = KC ? (KC | 1) : A.K1p;
  const size_t plane = (size_t)K2 * H;
  const int npair = (K2 + 1) / 2;
  const size_t bufsz = max(plane, (size_t)npair * K1p);
  float2* s0 = sm;
  float2* s1 = sm + bufsz;
  float2* tw1 = s1 + (pme_b_halves(KC) ? pme_b_half_w(KC) : bufsz);
  float2* tw2 = KC ? tw1 : tw1 + K1;  // one table for a cubic grid (K1 = K2)
  for (int i = threadIdx.x; i < (KC ? K1 : K1 + K2); i += blockDim.x) {
    const float2 t = A.twiddle[i];
    if (i < K1)
      tw1[i] = make_float2(t.x, -t.y);
    else
      tw2[i - K1] = make_float2(t.x, -t.y);
  }
  const float2* in = A.t1 + ((size_t)b * K3 + z) * plane;
  // k2 transforms, row-pair packing and the complex-to-real row transforms; res holds
  // the real rows, pair p (rows 2p, 2p + 1 interleaved) K1p apart
  float2* res = nullptr;
  if (live) {
    if constexpr (pme_b_halves(KC))
      res = pme_b_planes_halves<KC>(in, s0, s1, tw1);
    else if constexpr (KC > 0 && two_pass(KC) && KC % 4 == 0)
      res = pme_b_planes_fused<KC>(in, s0, s1, tw1);
    else
      res = pme_b_planes<KC>(A, in, s0, s1, tw1, tw2);
  }
  // padded periodic layout: grid point (x, y, z) lives at (x+h, y+h, z+h), h = P-1, and
  // the last h points of every axis are repeated below 0, so any stencil halo of the
  // gather is one in-bounds box (rows XP floats, planes YP rows, ZP planes)
  const int h = A.halo;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  // potential grids of 4 placements interleaved: phi[b/4][zp][yp][xp][b%4]
  float* out = A.phi + (size_t)(b >> 2) * A.ZP * A.YP * A.XP * 4 + (b & 3);
  const int KX = K1 + h, KY = K2 + h;  // written extent of a padded plane
  const int ncopy = (z >= K3 - h) ? 2 : 1;
  const float* resf = reinterpret_cast<const float*>(res);  // row pair p: (y = 2p, 2p+1) interleaved
  if constexpr (KC > 0) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ int sres_off;  // res within sm (float2 elements), -1 when the CTA has no placement
    if (threadIdx.x == 0) sres_off = live ? (int)(res - sm) : -1;
    cluster.sync();  // the four planes are complete and visible to the cluster
    const float2* rb[4];
    unsigned rlive = 0u;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int off = *cluster.map_shared_rank(&sres_off, k);
      if (off >= 0) rlive |= 1u << k;
      rb[k] = cluster.map_shared_rank(sm, k) + (off >= 0 ? off : 0);
    }
    // the lane's padded columns xx = lane + 32 i and their source columns, set up once
    constexpr int NX = (KC + 7 + 31) / 32;  // h <= 7
    int sx[NX];
    unsigned ok = 0u;
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      const int xx = lane + 32 * i;
      sx[i] = (xx < h) ? xx - h + KC : xx - h;
      if (xx < KX) ok |= 1u << i;
    }
    float4* grid4 = reinterpret_cast<float4*>(A.phi) + (size_t)blockIdx.z * A.ZP * A.YP * A.XP;
    const int rank = blockIdx.x;  // == the cluster rank (cluster dims (4, 1, 1))
    for (int c = 0; c < ncopy; ++c) {
      float4* plane_out = grid4 + (size_t)(c ? z - K3 + h : z + h) * A.YP * A.XP + lane;
      // one warp per row pair of this CTA's quarter (pairs rank, rank + 4, ...): one 8-byte
      // load per placement gives rows y = 2p (.x) and 2p + 1 (.y); row y is stored at
      // padded row y + h and, when y >= K2 - h, also at y + h - K2
      for (int pp = rank + 4 * warp; pp < npair; pp += 4 * nwarp) {
        const size_t prow = (size_t)pp * (KC | 1);
#pragma unroll
        for (int i = 0; i < NX; ++i) {
          if (!(ok & (1u << i))) continue;
          float2 v[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) v[k] = (rlive & (1u << k)) ? rb[k][prow + sx[i]] : make_float2(0.f, 0.f);
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int y = 2 * pp + e;
            if (y >= KC) break;
            const float4 q = e ? make_float4(v[0].y, v[1].y, v[2].y, v[3].y)
                               : make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
            plane_out[(size_t)(y + h) * A.XP + 32 * i] = q;
            if (y >= KC - h) plane_out[(size_t)(y + h - KC) * A.XP + 32 * i] = q;
          }
        }
      }
    }
    cluster.sync();  // no CTA leaves while another still reads its shared memory
  } else {
    for (int c = 0; c < ncopy; ++c) {
      float* plane_out = out + (size_t)(c ? z - K3 + h : z + h) * A.YP * A.XP * 4;
      for (int yy = warp; yy < KY; yy += nwarp) {  // one warp per padded row
        const int y = (yy < h) ? yy - h + K2 : yy - h;
        const float* src = resf + 2 * (size_t)(y >> 1) * K1p + (y & 1);
        float* dst = plane_out + (size_t)yy * A.XP * 4;
        for (int xx = lane; xx < KX; xx += 32) {
          const int x = (xx < h) ? xx - h + K1 : xx - h;
          dst[4 * xx] = src[2 * x];
        }
      }
    }
  }
}

// sized: the compile-time cubic kernel of this K runs (its work buffer may be a half one)
size_t pme_a_smem(int K3, int Hp, bool sized = false) {
  const size_t wcols = sized ? (size_t)pme_a_work_cols(K3) : (size_t)Hp;
  return sizeof(float2) * ((size_t)K3 * Hp + (size_t)K3 * wcols + K3);
}
// shared_tw: a cubic grid with compile-time sizes keeps one twiddle table for k1 and k2
size_t pme_b_smem(int K1, int K2, int H, bool shared_tw) {
  const size_t plane = (size_t)K2 * H;
  const size_t npair = (K2 + 1) / 2;
  const size_t bufsz = std::max(plane, npair * (size_t)(K1 | 1));
  // the compile-time cubic kernels of large grids keep one full buffer and a half one
  const size_t second = (shared_tw && pme_b_halves(K1)) ? pme_b_half_w(K1) : bufsz;
  return sizeof(float2) * (bufsz + second + K1 + (shared_tw ? 0 : K2));
}

}  // namespace

bool pme_fits(int K1, int K2, int K3) {
  const int H = K1 / 2 + 1, Hp = ((H + kR1 - 1) / kR1) * kR1;
  FftPlan a, b, c;
  if (!plan(K1, a) || !plan(K2, b) || !plan(K3, c)) return false;
  return pme_a_smem(K3, Hp) <= 227 * 1024 && pme_b_smem(K1, K2, H, false) <= 227 * 1024;
}

cudaError_t launch_pme_mixed(Engine& e, const BatchArgs& a) {
  PmeArgs A{};
  A.bvec = a.u_bvec;
  A.u_qf = a.u_qf;
  A.u_nsite = a.u_nsite;
  A.engfac = e.d_engfac_f;
  A.twiddle = e.d_twiddle;
  A.t1 = a.spec;
  A.phi = a.phi;
  A.self_part = a.self_part;
  A.nb = a.nb;
  A.K1 = e.geom.K[0];
  A.K2 = e.geom.K[1];
  A.K3 = e.geom.K[2];
  A.H = e.H();
  A.Hp = ((A.H + kR1 - 1) / kR1) * kR1;
  A.Kmax = e.Kmax();
  A.K1p = A.K1 | 1;
  A.halo = e.P_order - 1;
  A.XP = e.phi_dims[0];
  A.YP = e.phi_dims[1];
  A.ZP = e.phi_dims[2];
  if (!plan(A.K1, A.p1) || !plan(A.K2, A.p2) || !plan(A.K3, A.p3)) return cudaErrorInvalidValue;
  A.fH = make_fastdiv(A.H);
  A.fK1 = make_fastdiv(A.K1);
  A.fHp4 = make_fastdiv(A.Hp / kR1);
  A.fnpair = make_fastdiv((A.K2 + 1) / 2);
  A.fKX = make_fastdiv(A.K1 + A.halo);
  cudaError_t err;
  // cubic grids of common sizes take the compile-time transforms
  struct Sized {
    int K;
    void (*a)(PmeArgs);
    void (*b)(PmeArgs);
  };
#define ERMOD_PME_SIZE(KK) Sized{KK, pme_a_kernel<KK>, pme_b_kernel<KK>}
  static const Sized sized[] = {ERMOD_PME_SIZE(32),  ERMOD_PME_SIZE(40),  ERMOD_PME_SIZE(45),  ERMOD_PME_SIZE(48),
                                ERMOD_PME_SIZE(50),  ERMOD_PME_SIZE(60),  ERMOD_PME_SIZE(64),  ERMOD_PME_SIZE(72),
                                ERMOD_PME_SIZE(80),  ERMOD_PME_SIZE(90),  ERMOD_PME_SIZE(96),  ERMOD_PME_SIZE(100),
                                ERMOD_PME_SIZE(108), ERMOD_PME_SIZE(120), ERMOD_PME_SIZE(125), ERMOD_PME_SIZE(128),
                                ERMOD_PME_SIZE(144)};
#undef ERMOD_PME_SIZE
  constexpr int nsized = (int)(sizeof(sized) / sizeof(sized[0]));
  const bool cubic = A.K1 == A.K2 && A.K2 == A.K3;
  int slot = 0;  // 0: the generic kernels, 1 + i: sized[i]
  void (*ka)(PmeArgs) = pme_a_kernel<0>;
  void (*kb)(PmeArgs) = pme_b_kernel<0>;
  for (int i = 0; i < nsized && cubic; ++i)
    if (sized[i].K == A.K1) {
      slot = 1 + i;
      ka = sized[i].a;
      kb = sized[i].b;
    }
  const int KC = slot ? A.K1 : 0;
  // solute sites staged per generation chunk: both tables, chunk x (K3 + Hp), fit in pme_a's
  // work buffer
  const int wcols = KC ? pme_a_work_cols(KC) : A.Hp;
  A.chunk = std::max(1, std::min(kSites, (A.K3 * wcols) / (A.K3 + A.Hp)));
  const size_t sa = pme_a_smem(A.K3, A.Hp, KC > 0), sb = pme_b_smem(A.K1, A.K2, A.H, KC > 0);
  static SmemAttr attr_a[1 + nsized], attr_b[1 + nsized];  // per kernel
  if ((err = attr_a[slot].ensure(ka, sa)) != cudaSuccess) return err;
  if ((err = attr_b[slot].ensure(kb, sb)) != cudaSuccess) return err;
  const int nthr = pme_threads(KC);
  ka<<<dim3(A.K2, a.nb), nthr, sa, a.stream>>>(A);
  e.count_launch();
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  if (a.phases) {
    e.phase_end_on(a.stream);
    e.phase_begin_on(PH_FFT, a.stream);
  }
  if (slot) {  // compile-time sizes: the four CTAs of a group are one cluster
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(4, A.K3, (a.nb + 3) / 4);
    cfg.blockDim = dim3(nthr);
    cfg.dynamicSmemBytes = sb;
    cfg.stream = a.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 4;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if ((err = cudaLaunchKernelEx(&cfg, kb, A)) != cudaSuccess) return err;
  } else {
    kb<<<dim3(4, A.K3, (a.nb + 3) / 4), nthr, sb, a.stream>>>(A);
  }
  e.count_launch();
  return cudaGetLastError();
}

}  // namespace ermod
