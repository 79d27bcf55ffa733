// kernels_accum.cu -- update_histogram's accumulation (engproc.F90:758-856).
//
//   accumulate    one CTA per batch: solute self energy u0 (engproc.F90:711-733), its
//                 weight engnmfc (wgtslf / volcorrect, engproc.F90:772-796,871-887),
//                 engnorm/engsmpl/avslf, eself, minuv/maxuv, flceng and slnuv, and
//                 edens += engnmfc * insdst.  Every FP64 sum runs in placement order, as
//                 in the reference's sequential loop, so results are bit-reproducible.
//                 A batch in which any molecule failed a bin check is not accumulated.
//   ring_compact  per placement, the ascending list of occupied bins (bin, count).
//   ecorr_rows    ecorr(iduvp, iduv) += engnmfc * insdst(iduv) * insdst(iduvp)
//                 (engproc.F90:841-853) for the placements buffered in the ring: each
//                 CTA owns a few rows of the matrix in shared memory and walks the
//                 placements in order, touching only occupied (row, column) pairs; an
//                 exact int64 mirror sum insdst(i) insdst(j) is kept beside it.
#include <mutex>

#include "engine.cuh"

namespace ermod {

namespace {

struct AccArgs {
  BatchArgs a;
  int ntile, numslv, ermax, esmax, nself;
  int selfcal, wgtslf, soln, estype, rigid, mbin_mode;
  double temp, volume, volfac;  // volfac = pi Qtot^2 / beta^2 / V / 2 (volcorrect)
  double screen;                // residual_ene(slt, slt) = -(pi Q Q / beta / beta / V) / 2
  double stat_weight_system;
  int bare;      // cltype 0: no reciprocal self energy, no residual, volcorrect without its factor
  int ff_keys;   // the tile partials' min and max are ordered float-float keys (mixed path)
  double* scal;  // {engnorm, engsmpl, avslf, voffset, voffset_init, usreal, usreal_valid}
  double* edens;
  double* eself;
  double* slnuv;
  double* minuv;
  double* maxuv;
  const long long* eskey;
  int* ring_valid;  // [nb] entries of this batch in the ring
  double* ring_w;
  int slvmax;
  double* u0;      // [nb] solute self energies of the batch
  int* self_bin;   // [nb] eself bin (0-based) or -1
  DevStatus* status;
  // intermediate-state extension (solution mode), null when off
  const unsigned char* zmask;  // [ermax] 1 where the reference-solvent density is zero
  double* edintm;              // [ermax]
  double* uvintm;              // [numslv]
  double* iscal;               // {soln_total, soln_intm, norm_intm}
};

constexpr int kAccThreads = 256;
constexpr int kMaxBatch = 512;

// an error in this batch or an earlier one of the call; errors of later batches (already
// running on the other stream) do not stop this batch's accumulation.  The answer cannot
// change between the accumulation kernels of a batch: the earlier batches' kernels are
// complete by then and the error key only decreases.
__device__ __forceinline__ bool batch_failed(const AccArgs& A) {
  const volatile unsigned long long* ek = &A.status->err_key;
  const unsigned long long k = *ek;
  return k != kNoError && (long long)(k >> 36) < (long long)A.a.b0 + A.a.nb;
}

// fixed-order block sum: thread t adds elements t, t+256, ... in order, then a fixed tree
__device__ __forceinline__ double block_sum_fixed(double* red, const double* x, int n, int stride) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[(size_t)i * stride];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// one CTA per placement: self energy u0, the self-energy bin check, and the per-species
// tile partials reduced to flceng / min / max (written to tile slot 0)
__global__ void __launch_bounds__(kAccThreads) reduce_kernel(AccArgs A) {
  const BatchArgs& a = A.a;
  const int b = blockIdx.x;
  __shared__ double red[kAccThreads];
  const double self = A.bare ? 0.0 : block_sum_fixed(red, a.self_part + (size_t)b * A.nself, A.nself, 1);
  for (int sp = 0; sp < A.numslv; ++sp) {
    const double* base = a.part + ((size_t)b * A.ntile * A.numslv + sp) * 3;
    const int stride = A.numslv * 3;
    const double s = block_sum_fixed(red, base, A.ntile, stride);
    double mn = INFINITY, mx = -INFINITY;
    for (int t = threadIdx.x; t < A.ntile; t += blockDim.x) {
      const double* pt = base + (size_t)t * stride;
      if (A.ff_keys) {
        mn = fmin(mn, ff_key_to_double(reinterpret_cast<const long long*>(pt)[1]));
        mx = fmax(mx, ff_key_to_double(reinterpret_cast<const long long*>(pt)[2]));
      } else {
        mn = fmin(mn, pt[1]);
        mx = fmax(mx, pt[2]);
      }
    }
    red[threadIdx.x] = mn;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st) red[threadIdx.x] = fmin(red[threadIdx.x], red[threadIdx.x + st]);
      __syncthreads();
    }
    mn = red[0];
    __syncthreads();
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
      __syncthreads();
    }
    mx = red[0];
    __syncthreads();
    if (threadIdx.x == 0) {
      double* out = a.part + ((size_t)b * A.ntile * A.numslv + sp) * 3;  // tile slot 0
      out[0] = s;
      out[1] = mn;
      out[2] = mx;
      if (a.flceng_out) a.flceng_out[(size_t)(a.b0 + b) * A.numslv + sp] = s;
    }
  }
  if (threadIdx.x == 0 && a.skip && a.skip[b]) {  // rejected by check_mol_configuration
    A.u0[b] = 0.0;
    A.self_bin[b] = -1;
    if (a.uvengy_out) a.uvengy_out[(size_t)(a.b0 + b) * (A.slvmax + 1)] = 0.0;
  } else if (threadIdx.x == 0) {
    double usreal;
    if (A.rigid)
      usreal = (A.scal[6] != 0.0) ? A.scal[5] : a.u_usreal[0];
    else
      usreal = a.u_usreal[b];
    const double qm = a.u_qmol[b];
    double epcl = A.bare ? 0.0 : kPi * qm * qm / A.screen / A.screen / A.volume;
    epcl = epcl / 2.0;
    const double residual = -epcl;
    double u0 = self;
    u0 = u0 + usreal + residual;  // uvengy(0) = uvengy(0) + pairep + residual
    A.u0[b] = u0;
    A.self_bin[b] = -1;
    if (a.uvengy_out) a.uvengy_out[(size_t)(a.b0 + b) * (A.slvmax + 1)] = u0;
    if (A.selfcal) {  // getiduv(0, uvengy(0))
      int code = 0, ret = 0;
      if (u0 != u0) {
        code = ERMOD_E_ENG_MIN;
      } else {
        const long long ku = ordered_key(u0);
        int lo = 0, hi = A.esmax;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (A.eskey[mid] < ku)
            lo = mid + 1;
          else
            hi = mid;
        }
        ret = lo;
        if (ret <= 0)
          code = ERMOD_E_ENG_MIN;
        else if (ret == A.esmax && u0 < 1.0e3 && A.mbin_mode != 0) {
          if (A.mbin_mode == 1)
            code = ERMOD_W_MBIN;
          else
            atomicOr(&A.status->mbin_hit, 1);
        }
      }
      if (code)
        atomicMin(&A.status->err_key, make_err_key(a.b0 + b, 0, code));
      else
        A.self_bin[b] = ret - 1;
    }
  }
}

__global__ void __launch_bounds__(kAccThreads) accumulate_kernel(AccArgs A) {
  const BatchArgs& a = A.a;
  const int nb = a.nb;
  __shared__ double sw[kMaxBatch];
  __shared__ double stw[kMaxBatch];
  __shared__ double su0[kMaxBatch];
  __shared__ int sbin[kMaxBatch];
  __shared__ double sterm[kMaxBatch];
  __shared__ double sred[2][kAccThreads];
  __shared__ unsigned char srej[kMaxBatch];  // rejected by the configuration check
  __shared__ int skip;
  __shared__ double s_voffset;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) srej[b] = (a.skip && a.skip[b]) ? 1 : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    skip = batch_failed(A) ? 1 : 0;
    if (!skip && A.wgtslf && A.scal[4] == 0.0) {
      // voffset from the first placement ever accumulated (update_histogram,
      // engproc.F90:779-783); rejected placements never reach it
      int first = 0;
      while (first < nb && srej[first]) ++first;
      if (first < nb) {
        A.scal[3] = A.u0[first];
        A.scal[4] = 1.0;
      }
    }
    if (!skip && A.rigid && A.scal[6] == 0.0) {
      A.scal[5] = a.u_usreal[0];
      A.scal[6] = 1.0;
    }
    s_voffset = A.scal[3];
  }
  __syncthreads();
  if (skip) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      a.engnmfc[b] = 0.0;
      A.ring_valid[b] = 0;
    }
    return;
  }
  // weights (parallel); u0 and the eself bins staged for the ordered sums
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    su0[b] = A.u0[b];
    sbin[b] = A.self_bin[b];
    if (srej[b]) {  // the loop's skipcond (engproc.F90:389-390): no update_histogram
      sw[b] = 0.0;
      stw[b] = 0.0;
      a.engnmfc[b] = 0.0;
      A.ring_w[b] = 0.0;
      A.ring_valid[b] = 0;
      continue;
    }
    double engnmfc;
    if (!A.wgtslf) {
      engnmfc = 1.0;
    } else {
      const double factor = su0[b] - s_voffset;
      engnmfc = A.soln ? exp(factor / A.temp) : exp(-factor / A.temp);
    }
    double total_weight = A.stat_weight_system * (a.stat_weight_solute ? a.stat_weight_solute[b] : 1.0);
    if (A.estype == 2) {
      total_weight = total_weight * A.volume;
      total_weight = total_weight * exp(A.volfac / A.temp);
    }
    engnmfc = engnmfc * total_weight;
    sw[b] = engnmfc;
    stw[b] = total_weight;
    a.engnmfc[b] = engnmfc;
    A.ring_w[b] = engnmfc;
    A.ring_valid[b] = 1;
  }
  __syncthreads();
  // ordered scalar sums (placement order, as the reference's loop)
  if (threadIdx.x == 0) {
    double engnorm = A.scal[0], engsmpl = A.scal[1], avslf = A.scal[2];
    double mn = A.minuv[0], mx = A.maxuv[0];
    for (int b = 0; b < nb; ++b) {
      if (srej[b]) continue;
      engnorm = engnorm + sw[b];
      engsmpl = engsmpl + 1.0;
      avslf = avslf + stw[b];
      if (A.selfcal) A.eself[sbin[b]] += sw[b];
      mn = fmin(mn, su0[b]);
      mx = fmax(mx, su0[b]);
    }
    A.scal[0] = engnorm;
    A.scal[1] = engsmpl;
    A.scal[2] = avslf;
    A.minuv[0] = mn;
    A.maxuv[0] = mx;
  }
  // per species: min/max over the batch (order-free tree), slnuv in placement order
  for (int sp = 0; sp < A.numslv; ++sp) {
    double mn = INFINITY, mx = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      const double* pt = a.part + ((size_t)b * A.ntile * A.numslv + sp) * 3;
      mn = fmin(mn, pt[1]);
      mx = fmax(mx, pt[2]);
      if (A.soln) sterm[b] = pt[0] * sw[b];
    }
    sred[0][threadIdx.x] = mn;
    sred[1][threadIdx.x] = mx;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st) {
        sred[0][threadIdx.x] = fmin(sred[0][threadIdx.x], sred[0][threadIdx.x + st]);
        sred[1][threadIdx.x] = fmax(sred[1][threadIdx.x], sred[1][threadIdx.x + st]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      A.minuv[sp + 1] = fmin(A.minuv[sp + 1], sred[0][0]);
      A.maxuv[sp + 1] = fmax(A.maxuv[sp + 1], sred[1][0]);
      if (A.soln) {
        double sl = A.slnuv[sp];
        for (int b = 0; b < nb; ++b)
          if (!srej[b]) sl = sl + sterm[b];
        A.slnuv[sp] = sl;
      }
    }
    __syncthreads();
  }
  if (!A.zmask) return;  // edens: accumulate_bins_kernel
  // edens += engnmfc * insdst, placements in order
  for (int i = threadIdx.x; i < A.ermax; i += blockDim.x) {
    double e = A.edens[i];
    bool touched = false;
    for (int b = 0; b < nb; ++b) {
      const int c = a.hist[(size_t)b * A.ermax + i];
      if (c) {
        e = e + sw[b] * (double)c;
        touched = true;
      }
    }
    if (touched) A.edens[i] = e;
  }
  // intermediate state (extensions/Intermediate/engproc.F90, update_histogram hunk):
  // a placement belongs to it when none of its occupied bins has zero density in the
  // reference solvent; its weight, histogram and flceng then accumulate separately
  if (A.zmask) {
    __shared__ unsigned char sout[kMaxBatch];
    for (int b = 0; b < nb; ++b) {
      int out = 0;
      for (int i = threadIdx.x; i < A.ermax; i += blockDim.x)
        if (A.zmask[i] && a.hist[(size_t)b * A.ermax + i] > 0) out = 1;
      out = __syncthreads_or(out);
      if (threadIdx.x == 0) sout[b] = (unsigned char)out;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = A.iscal[0], in = A.iscal[1], nrm = A.iscal[2];
      for (int b = 0; b < nb; ++b) {
        if (srej[b]) continue;
        tot = tot + sw[b];
        if (!sout[b]) {
          in = in + sw[b];
          nrm = nrm + sw[b];
        }
      }
      A.iscal[0] = tot;
      A.iscal[1] = in;
      A.iscal[2] = nrm;
    }
    for (int i = threadIdx.x; i < A.ermax; i += blockDim.x) {
      double e = A.edintm[i];
      for (int b = 0; b < nb; ++b) {
        const int c = a.hist[(size_t)b * A.ermax + i];
        if (c > 0 && !sout[b]) e = e + sw[b] * (double)c;
      }
      A.edintm[i] = e;
    }
    for (int sp = threadIdx.x; sp < A.numslv; sp += blockDim.x) {
      double u = A.uvintm[sp];
      for (int b = 0; b < nb; ++b)
        if (!sout[b]) u = u + a.part[((size_t)b * A.ntile * A.numslv + sp) * 3] * sw[b];
      A.uvintm[sp] = u;
    }
  }
}

// edens += engnmfc * insdst (engproc.F90:836-838), one thread per bin, the batch's
// placements in order (so the FP64 sums are those of the reference's loop); the
// intermediate-state mode does this inside accumulate_kernel instead
__global__ void __launch_bounds__(128) accumulate_bins_kernel(AccArgs A) {
  const BatchArgs& a = A.a;
  const int nb = a.nb;
  if (nb <= 0 || batch_failed(A)) return;  // the batch was not accumulated (an error)
  __shared__ double sw[kMaxBatch];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sw[b] = a.engnmfc[b];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.ermax) return;
  const int* h = a.hist + i;
  const size_t E = (size_t)A.ermax;
  double e = A.edens[i];
  bool touched = false;
  int b = 0;
  for (; b + 8 <= nb; b += 8) {
    int c[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) c[u] = __ldg(h + (size_t)(b + u) * E);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (c[u]) {
        e = e + sw[b + u] * (double)c[u];
        touched = true;
      }
  }
  for (; b < nb; ++b) {
    const int c = __ldg(h + (size_t)b * E);
    if (c) {
      e = e + sw[b] * (double)c;
      touched = true;
    }
  }
  if (touched) A.edens[i] = e;
}

// occupied-bin list per ring entry: entries (bin << 0) with counts beside them
__global__ void __launch_bounds__(256) ring_compact_kernel(const int* __restrict__ hist, const int* __restrict__ valid,
                                                         int ermax, int* __restrict__ nz_bin, int* __restrict__ nz_cnt,
                                                         int* __restrict__ nnz) {
  const int p = blockIdx.x;
  const int* h = hist + (size_t)p * ermax;
  __shared__ int scan[256];
  const int per = (ermax + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(ermax, lo + per);
  int cnt = 0;
  if (valid[p])
    for (int i = lo; i < hi; ++i) cnt += (h[i] != 0);
  scan[threadIdx.x] = cnt;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {  // inclusive Hillis-Steele scan
    const int v = (threadIdx.x >= off) ? scan[threadIdx.x - off] : 0;
    __syncthreads();
    scan[threadIdx.x] += v;
    __syncthreads();
  }
  int pos = scan[threadIdx.x] - cnt;
  if (valid[p])
    for (int i = lo; i < hi; ++i)
      if (h[i]) {
        nz_bin[(size_t)p * ermax + pos] = i;
        nz_cnt[(size_t)p * ermax + pos] = h[i];
        ++pos;
      }
  if (threadIdx.x == blockDim.x - 1) nnz[p] = valid[p] ? scan[threadIdx.x] : 0;
}

__global__ void __launch_bounds__(256) ecorr_rows_kernel(const int* __restrict__ hist, const int* __restrict__ nz_bin,
                                                       const int* __restrict__ nz_cnt, const int* __restrict__ nnz,
                                                       const double* __restrict__ w, int nring, int ermax, int R,
                                                       double* __restrict__ ecorr, long long* __restrict__ ecorr_n) {
  extern __shared__ double srow[];  // [R][ermax] (+ [R][ermax] int64 mirror)
  long long* srow_n = reinterpret_cast<long long*>(srow + (size_t)R * ermax);
  const int row0 = blockIdx.x * R;
  const int nrow = min(R, ermax - row0);
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int t = threadIdx.x; t < nring * nrow; t += blockDim.x) {
    const int p = t / nrow, r = t % nrow;
    if (nnz[p] > 0 && hist[(size_t)p * ermax + row0 + r] != 0) any = 1;
  }
  __syncthreads();
  if (!any) return;
  for (int t = threadIdx.x; t < nrow * ermax; t += blockDim.x) {
    srow[t] = ecorr[(size_t)row0 * ermax + t];
    if (ecorr_n) srow_n[t] = ecorr_n[(size_t)row0 * ermax + t];
  }
  __syncthreads();
  for (int p = 0; p < nring; ++p) {
    const int n = nnz[p];
    if (n == 0) continue;
    const int* bins = nz_bin + (size_t)p * ermax;
    const int* cnts = nz_cnt + (size_t)p * ermax;
    for (int r = 0; r < nrow; ++r) {
      const int ci = hist[(size_t)p * ermax + row0 + r];
      if (ci == 0) continue;
      const double wi = w[p] * (double)ci;
      double* row = srow + (size_t)r * ermax;
      long long* rown = srow_n + (size_t)r * ermax;
      for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int j = bins[t];
        const int cj = cnts[t];
        row[j] = row[j] + wi * (double)cj;
        if (ecorr_n) rown[j] += (long long)ci * (long long)cj;
      }
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nrow * ermax; t += blockDim.x) {
    ecorr[(size_t)row0 * ermax + t] = srow[t];
    if (ecorr_n) ecorr_n[(size_t)row0 * ermax + t] = srow_n[t];
  }
}

// the dynamic shared memory of ecorr_rows_kernel, shared by the FP64 flush and the
// no-allocation entry point: one record, so that a caller needing less never lowers the
// size another caller has set
SmemAttr& ecorr_rows_attr() {
  static SmemAttr attr;
  return attr;
}

// Mixed path flush, same sum as ecorr_rows_kernel.  A CTA owns kEcRows rows and 256
// columns of the matrix; thread t owns one column and keeps the flush's contribution
// to its kEcRows entries in registers as float-float pairs (exact products by fma,
// TwoSum additions: ~44 significant bits), walking the ring's placements in order.
// No two threads share an entry, so the walk needs no barrier and its loads pipeline;
// the pairs are added to the FP64 matrix once per flush.  The row coefficients
// hist[p][row0 + r] of every placement are staged in shared memory with a bit mask of
// the nonzero ones.
constexpr int kEcRows = 8;

__device__ __forceinline__ void ff_add_prod(float& hi, float& lo, float wh, float wl, float c) {
  const float p = wh * c;
  float pe = fmaf(wh, c, -p);  // exact low part of wh * c
  pe = fmaf(wl, c, pe);
  const float s = hi + p;  // TwoSum(hi, p)
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (p - bb);
  lo += err + pe;
  hi = s;
}

// The rows and columns walked are the flush's active bins only (act[0 .. *nact): the bins
// some placement of the ring occupies, in increasing order), so a coordinate of thousands
// of bins costs what its occupied part costs; an inactive row or column has no
// contribution, so the sums are those of the walk over every bin.  The matrix is
// symmetric: only entries on or above the diagonal (column index >= row index in act) are
// summed, and each is added at (row, column) and (column, row), so that both halves get
// the same value from one sum.
template <bool COUNT>
__global__ void __launch_bounds__(256, 2) ecorr_ff_kernel(const int* __restrict__ hist, const int* __restrict__ valid,
                                                        const double* __restrict__ w, int nring, int ermax,
                                                        const int* __restrict__ act, const int* __restrict__ nact_d,
                                                        double* __restrict__ ecorr, long long* __restrict__ ecorr_n) {
  extern __shared__ float2 sdyn2[];
  float2* sa = sdyn2;  // [nring][kEcRows]: w_p * hist[p][row r's bin] as a float-float pair
  unsigned* smask = reinterpret_cast<unsigned*>(sa + (size_t)nring * kEcRows);  // [nring]
  int* sci = reinterpret_cast<int*>(smask + nring);  // [nring][kEcRows] counts (count mirror only)
  const int nact = *nact_d;
  const int row0 = blockIdx.y * kEcRows;
  if (row0 >= nact) return;  // the grid covers every bin; the active ones come first
  if ((int)(blockIdx.x * blockDim.x + blockDim.x) <= row0) return;  // all below the diagonal
  const int nrow = min(kEcRows, nact - row0);
  int rbin[kEcRows];
#pragma unroll
  for (int r = 0; r < kEcRows; ++r) rbin[r] = act[row0 + min(r, nrow - 1)];
  const int jj = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = jj < nact ? act[jj] : ermax;  // this thread's column (ermax: none)
  for (int p = threadIdx.x; p < nring; p += blockDim.x) {
    unsigned m = 0;
    const bool ok = valid[p] != 0;
    const double wd = w[p];
    const float wh = (float)wd;
    const float wl = (float)(wd - (double)wh);
    for (int r = 0; r < kEcRows; ++r) {
      const int c = (ok && r < nrow) ? hist[(size_t)p * ermax + rbin[r]] : 0;
      // w * c as a float-float pair (c < 2^24 is exact in FP32; the high product is
      // split exactly by fma)
      const float fc = (float)c;
      const float ah = wh * fc;
      const float al = fmaf(wl, fc, fmaf(wh, fc, -ah));
      sa[p * kEcRows + r] = make_float2(ah, al);
      if (COUNT) sci[p * kEcRows + r] = c;
      if (c) m |= 1u << r;
    }
    smask[p] = m;
  }
  __syncthreads();
  if (j >= ermax || jj < row0) return;
  // rows r <= jj - row0 of this column are on or above the diagonal
  const unsigned rows_on = (jj - row0 >= kEcRows - 1) ? 0xffu : ((2u << (jj - row0)) - 1u);
  float hi[kEcRows], lo[kEcRows];
  long long cn[COUNT ? kEcRows : 1];
#pragma unroll
  for (int r = 0; r < kEcRows; ++r) {
    hi[r] = 0.f;
    lo[r] = 0.f;
    if (COUNT) cn[r] = 0;
  }
  bool any = false;
  constexpr int U = 4;  // loads in flight per thread
  for (int p0 = 0; p0 < nring; p0 += U) {
    int cj[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = p0 + u;
      cj[u] = (p < nring && smask[p]) ? __ldg(hist + (size_t)p * ermax + j) : 0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (cj[u] == 0) continue;
      const int p = p0 + u;
      any = true;
      const unsigned m = smask[p] & rows_on;
      const float c = (float)cj[u];
      const float2* ap = sa + p * kEcRows;
#pragma unroll
      for (int r = 0; r < kEcRows; ++r) {
        if (m & (1u << r)) {
          const float2 a = ap[r];
          ff_add_prod(hi[r], lo[r], a.x, a.y, c);
          if (COUNT) cn[r] += (long long)sci[p * kEcRows + r] * (long long)cj[u];
        }
      }
    }
  }
  if (!any) return;
#pragma unroll
  for (int r = 0; r < kEcRows; ++r) {
    if (r >= nrow) break;
    const size_t at = (size_t)rbin[r] * ermax + j, ta = (size_t)j * ermax + rbin[r];
    if (hi[r] != 0.f || lo[r] != 0.f) {
      const double v = (double)hi[r] + (double)lo[r];
      ecorr[at] = ecorr[at] + v;
      if (ta != at) ecorr[ta] = ecorr[ta] + v;
    }
    if (COUNT && cn[r] != 0) {
      ecorr_n[at] += cn[r];
      if (ta != at) ecorr_n[ta] += cn[r];
    }
  }
}

// The flush's active bins: flag[i] != 0 when some valid placement of the ring occupies bin
// i (flag zeroed first).  CTA per (256 bins, 32 placements): the 32 loads of a thread are
// independent and in flight together; an occupied bin sets its flag (an OR, so the
// order of the writes does not matter).
constexpr int kActivePlacements = 32;
__global__ void __launch_bounds__(256) ring_active_kernel(const int* __restrict__ hist, const int* __restrict__ valid,
                                                        int nring, int ermax, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int p0 = blockIdx.y * kActivePlacements;
  if (i >= ermax) return;
  int c[kActivePlacements];
#pragma unroll
  for (int u = 0; u < kActivePlacements; ++u) {
    const int p = p0 + u;
    c[u] = (p < nring && valid[p]) ? __ldg(hist + (size_t)p * ermax + i) : 0;
  }
  int any = 0;
#pragma unroll
  for (int u = 0; u < kActivePlacements; ++u) any |= c[u];
  if (any) flag[i] = 1;
}

// Coordinates of at most this many bins walk every bin: on the 33,000-water workload
// (1,396 bins, about 900 of them active in a flush) the gathered walk over the active
// ones was slower than the contiguous walk over all.
constexpr int kActiveMinBins = 2048;

// act[0 .. *nact) = the flagged bins in increasing order (one CTA, chunks of 1024)
__global__ void __launch_bounds__(1024) ring_active_list_kernel(const int* __restrict__ flag, int ermax,
                                                              int* __restrict__ act, int* __restrict__ nact) {
  __shared__ int scan[1024];
  int base = 0;
  for (int c0 = 0; c0 < ermax; c0 += 1024) {
    const int i = c0 + (int)threadIdx.x;
    const int f = (i < ermax && flag[i] != 0) ? 1 : 0;
    scan[threadIdx.x] = f;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
      const int v = (threadIdx.x >= (unsigned)off) ? scan[threadIdx.x - off] : 0;
      __syncthreads();
      scan[threadIdx.x] += v;
      __syncthreads();
    }
    if (f) act[base + scan[threadIdx.x] - 1] = i;
    const int tot = scan[1023];
    __syncthreads();  // scan[1023] read by every thread before the next chunk overwrites it
    base += tot;
  }
  if (threadIdx.x == 0) *nact = base;
}

}  // namespace

int accumulate_max_batch() { return kMaxBatch; }

cudaError_t launch_accumulate(Engine& e, const BatchArgs& a, cudaStream_t s) {
  AccArgs A{};
  A.a = a;
  A.ntile = e.ntile;
  A.numslv = e.numslv;
  A.ermax = e.ermax;
  A.esmax = e.esmax;
  A.nself = e.mixed ? spectrum_partials(e) : influence64_blocks();
  A.selfcal = e.P.selfcal;
  A.wgtslf = e.P.wgtslf;
  A.soln = e.P.slttype == 1;
  A.estype = e.P.estype;
  A.rigid = e.P.slttype == 2;
  A.mbin_mode = e.warn_bin_firsttime ? (e.P.force_calculation ? 2 : 1) : 0;
  A.temp = e.P.temp;
  A.volume = e.geom.volume;
  A.bare = (e.P.cltype == 0) ? 1 : 0;
  A.ff_keys = e.mixed ? 1 : 0;
  A.volfac = A.bare ? 0.0  // volcorrect multiplies by the volume only (engproc.F90:871-887)
                    : kPi * (e.total_charge_phys * e.total_charge_phys) / (e.P.screen * e.P.screen) / e.geom.volume / 2.0;
  A.screen = e.P.screen;
  A.stat_weight_system = e.stat_weight_system;
  A.scal = e.d_scal;
  A.edens = e.d_edens;
  A.eself = e.d_eself;
  A.slnuv = e.d_slnuv;
  A.minuv = e.d_minuv;
  A.maxuv = e.d_maxuv;
  A.eskey = e.d_eskey;
  A.ring_valid = e.d_ring_valid + e.ring_off + e.ring_fill;
  A.ring_w = e.d_ring_w + e.ring_off + e.ring_fill;
  A.slvmax = e.slvmax;
  A.u0 = a.u0;
  A.self_bin = a.self_bin;
  A.status = e.d_status;
  if (e.d_int_mask) {
    A.zmask = e.d_int_mask;
    A.edintm = e.d_edintm;
    A.uvintm = e.d_edintm + e.ermax;
    A.iscal = e.d_edintm + e.ermax + e.numslv;
  }
  reduce_kernel<<<a.nb, kAccThreads, 0, s>>>(A);
  accumulate_kernel<<<1, kAccThreads, 0, s>>>(A);
  e.count_launch(2);
  if (!A.zmask) {
    accumulate_bins_kernel<<<(e.ermax + 127) / 128, 128, 0, s>>>(A);
    e.count_launch();
  }
  return cudaGetLastError();
}

cudaError_t launch_ecorr_flush(Engine& e, cudaStream_t s) {
  if (e.ring_fill == 0) return cudaSuccess;
  const int n = e.ring_fill;
  if (e.mixed) {
    const bool count = e.d_ecorr_n != nullptr;
    const size_t smem =
        (size_t)n * (kEcRows * sizeof(float2) + sizeof(unsigned) + (count ? kEcRows * sizeof(int) : 0));
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    const int* hist = e.d_ring_hist + (size_t)e.ring_off * e.ermax;
    const int* valid = e.d_ring_valid + e.ring_off;
    int* flag = e.d_ring_nz;                  // [ermax] occupied by some placement
    int* act = e.d_ring_nz + e.ermax;         // [ermax] the active bins
    int* nact = e.d_ring_nz + 2 * e.ermax;    // [1]
    if (e.ermax > kActiveMinBins) {
      if ((err = cudaMemsetAsync(flag, 0, sizeof(int) * e.ermax, s)) != cudaSuccess) return err;
      ring_active_kernel<<<dim3((e.ermax + 255) / 256, (n + kActivePlacements - 1) / kActivePlacements), 256, 0, s>>>(
          hist, valid, n, e.ermax, flag);
    } else {  // every bin walked: the list costs more than the bins it could leave out
      if ((err = cudaMemsetAsync(flag, 0xff, sizeof(int) * e.ermax, s)) != cudaSuccess) return err;
    }
    ring_active_list_kernel<<<1, 1024, 0, s>>>(flag, e.ermax, act, nact);
    e.count_launch(e.ermax > kActiveMinBins ? 2 : 1);
    void (*kern)(const int*, const int*, const double*, int, int, const int*, const int*, double*, long long*) =
        count ? ecorr_ff_kernel<true> : ecorr_ff_kernel<false>;
    static SmemAttr attr_ff[2];  // per instantiation; the size set only ever grows
    if ((err = attr_ff[count ? 1 : 0].ensure(kern, smem)) != cudaSuccess) return err;
    dim3 grid((e.ermax + 255) / 256, (e.ermax + kEcRows - 1) / kEcRows);
    kern<<<grid, 256, smem, s>>>(hist, valid, e.d_ring_w + e.ring_off, n, e.ermax, act, nact, e.d_ecorr, e.d_ecorr_n);
    e.count_launch();
    return cudaGetLastError();
  }
  int* nz_bin = e.d_ring_nz;
  int* nz_cnt = e.d_ring_nz + (size_t)e.ring_cap * e.ermax;
  const int* valid = e.d_ring_valid + e.ring_off;
  const int* hist = e.d_ring_hist + (size_t)e.ring_off * e.ermax;
  ring_compact_kernel<<<n, 256, 0, s>>>(hist, valid, e.ermax, nz_bin, nz_cnt, e.d_ring_nnz);
  e.count_launch();
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const size_t per_row = (size_t)e.ermax * (sizeof(double) + (e.d_ecorr_n ? sizeof(long long) : 0));
  int R = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024) / per_row));
  const size_t smem = per_row * R;
  if ((err = ecorr_rows_attr().ensure(ecorr_rows_kernel, smem)) != cudaSuccess) return err;
  const int nblk = (e.ermax + R - 1) / R;
  ecorr_rows_kernel<<<nblk, 256, smem, s>>>(hist, nz_bin, nz_cnt, e.d_ring_nnz, e.d_ring_w + e.ring_off, n,
                                                   e.ermax, R, e.d_ecorr, e.d_ecorr_n);
  e.count_launch();
  return cudaGetLastError();
}


// ---- ecorr from caller-owned histograms, with no allocation -----------------------
//
// Some hosts cannot let a library allocate device memory in the middle of their step:
// an MD engine that has sized its memory pool to the whole card, or one that keeps
// other streams busy on the same device, where cudaFree would synchronise the device
// and stall them.  ermod_ecorr_add_noalloc serves such hosts.  Its only scratch (the
// occupied-bin lists that ring_compact_kernel builds for the ring) lives in one fixed
// file-scope device array, so a call allocates nothing.

namespace {

constexpr size_t kNoAllocEntries = (size_t)kNoAllocMaxEntries;  // 8 MiB of (bin, count) lists
constexpr int kNoAllocMaxDevices = 64;

// [kNoAllocEntries] bins, [kNoAllocEntries] counts, [kNoAllocMaxPlace] list lengths.
// Shared by every call on a device: calls that overlap on the GPU race on it.
static __device__ __align__(256) int g_noalloc_scratch[2 * kNoAllocEntries + kNoAllocMaxPlace];

std::mutex g_noalloc_mu;
int* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// ring_compact_kernel for caller histograms: every placement is valid, the lists go to
// the fixed scratch.  Each list length is written for every placement and each list
// entry below it, so nothing in the scratch has to start at zero.
__global__ void __launch_bounds__(256) compact_noalloc_kernel(const int* __restrict__ hist, int ermax,
                                                              int* __restrict__ nz_bin, int* __restrict__ nz_cnt,
                                                              int* __restrict__ nnz) {
  const int p = blockIdx.x;
  const int* h = hist + (size_t)p * ermax;
  __shared__ int scan[256];
  const int per = (ermax + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(ermax, lo + per);
  int cnt = 0;
  for (int i = lo; i < hi; ++i) cnt += (h[i] != 0);
  scan[threadIdx.x] = cnt;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    const int v = (threadIdx.x >= off) ? scan[threadIdx.x - off] : 0;
    __syncthreads();
    scan[threadIdx.x] += v;
    __syncthreads();
  }
  int pos = scan[threadIdx.x] - cnt;
  for (int i = lo; i < hi; ++i)
    if (h[i]) {
      nz_bin[(size_t)p * ermax + pos] = i;
      nz_cnt[(size_t)p * ermax + pos] = h[i];
      ++pos;
    }
  if (threadIdx.x == blockDim.x - 1) nnz[p] = scan[threadIdx.x];
}

// the scratch address on the current device, looked up once per device
cudaError_t noalloc_scratch(int** out) {
  int dev = -1;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    int* p = nullptr;
    err = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (err != cudaSuccess) return err;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_ecorr_noalloc(const int* hist, const double* weight, int nplace, int ermax, double* ecorr,
                                 long long* ecorr_count, cudaStream_t s) {
  int* scratch = nullptr;
  cudaError_t err = noalloc_scratch(&scratch);
  if (err != cudaSuccess) return err;
  int* nz_bin = scratch;
  int* nz_cnt = scratch + kNoAllocEntries;
  int* nnz = scratch + 2 * kNoAllocEntries;
  compact_noalloc_kernel<<<nplace, 256, 0, s>>>(hist, ermax, nz_bin, nz_cnt, nnz);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const size_t per_row = (size_t)ermax * (sizeof(double) + (ecorr_count ? sizeof(long long) : 0));
  const int R = (int)std::max<size_t>(1, std::min<size_t>(8, (96 * 1024) / per_row));
  const size_t smem = per_row * R;
  err = ecorr_rows_attr().ensure(ecorr_rows_kernel, smem);
  if (err != cudaSuccess) return err;
  ecorr_rows_kernel<<<(ermax + R - 1) / R, 256, smem, s>>>(hist, nz_bin, nz_cnt, nnz, weight, nplace, ermax, R,
                                                           ecorr, ecorr_count);
  return cudaGetLastError();
}

}  // namespace ermod
