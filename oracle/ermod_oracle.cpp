// ermod_oracle.cpp -- FP64 CPU restatement of ERmod's energy-representation hot path.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU baseline.
// The product never links or calls this file.  Parity status: partially pinned (the
// reference's own golden vectors exist only for spline_value, spline_test.F90:19-40;
// everything else is pinned by analytic checks, see ermod_oracle.h).
//
// Every routine cites the reference routine it restates (file:line within ERmod).
// Arithmetic order follows the Fortran source where it matters for rounding
// (products inside the spline/spread/gather loops, the bin-edge construction).
// Deviations, all at the 1e-15 relative level:
//   * the 3-D FFT is written here (mixed radix) instead of FFTW/MKL;
//   * normalize_periodic's LAPACK QR is omitted: for the cuboid cells the reference
//     accepts (realcal.F90:859-866) it is the identity up to an axis permutation,
//     so the wrap into [0, L) is done directly;
//   * OpenMP splits the placement loop over threads (each placement's energies are
//     computed by one thread), then update_histogram runs in placement order, so the
//     accumulators are bit-identical to a sequential run.
#include "ermod_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
constexpr double PI = 3.1415926535897932;  // engmain.F90:250
constexpr double INFTY = 1.0e50;           // engproc.F90:56

// ---------------------------------------------------------------------------------
// Mixed-radix complex FFT (recursive decimation in time), written for this oracle.
// Replaces the FFTW / MKL DFTI calls of fft_iface.F90:116-141,204-226.
// ---------------------------------------------------------------------------------
struct Fft1d {
  int n = 0;
  std::vector<int> fac;
  std::vector<cd> tw;  // tw[j] = exp(-2 pi i j / n)

  void init(int n_) {
    n = n_;
    fac.clear();
    int m = n;
    for (int p : {4, 2, 3, 5}) {
      while (m % p == 0) {
        fac.push_back(p);
        m /= p;
      }
    }
    for (int p = 7; m > 1; p += 2) {
      while (m % p == 0) {
        fac.push_back(p);
        m /= p;
      }
    }
    tw.resize(n);
    for (int j = 0; j < n; ++j) {
      // exact values on the axes, long double elsewhere
      if ((4 * (int64_t)j) % n == 0) {
        int q = (int)((4 * (int64_t)j) / n);
        const double c[4] = {1.0, 0.0, -1.0, 0.0}, s[4] = {0.0, -1.0, 0.0, 1.0};
        tw[j] = cd(c[q], s[q]);
      } else {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)j / (long double)n;
        tw[j] = cd((double)cosl(a), (double)sinl(a));
      }
    }
  }

  inline cd w(int64_t j, int sign) const {
    const cd& t = tw[(size_t)(j % n)];
    return sign < 0 ? t : std::conj(t);
  }

  void rec(const cd* in, int is, cd* out, int len, int fi, int sign) const {
    if (len == 1) {
      out[0] = in[0];
      return;
    }
    const int p = fac[fi], m = len / p;
    for (int q = 0; q < p; ++q) rec(in + (size_t)q * is, is * p, out + (size_t)q * m, m, fi + 1, sign);
    const int step = n / len;
    cd t[64];
    for (int k = 0; k < m; ++k) {
      for (int q = 0; q < p; ++q) t[q] = (q == 0 || k == 0) ? out[(size_t)q * m + k] : out[(size_t)q * m + k] * w((int64_t)q * k * step, sign);
      if (p == 2) {
        out[k] = t[0] + t[1];
        out[m + k] = t[0] - t[1];
      } else if (p == 4) {
        const cd a = t[0] + t[2], b = t[0] - t[2], c = t[1] + t[3];
        cd d = t[1] - t[3];
        d = sign < 0 ? cd(d.imag(), -d.real()) : cd(-d.imag(), d.real());  // d * (-+i)
        out[k] = a + c;
        out[m + k] = b + d;
        out[2 * m + k] = a - c;
        out[3 * m + k] = b - d;
      } else {
        for (int r = 0; r < p; ++r) {
          cd acc = t[0];
          for (int q = 1; q < p; ++q) acc += t[q] * w((int64_t)q * r * m * step, sign);
          out[(size_t)r * m + k] = acc;
        }
      }
    }
  }
  // out[k] = sum_j in[j*is] exp(sign 2 pi i j k / n)
  void exec(const cd* in, int is, cd* out, int sign) const { rec(in, is, out, n, 0, sign); }
};

struct Fft3d {
  int k1 = 0, k2 = 0, k3 = 0, h = 0;
  Fft1d f1, f2, f3;
  void init(int a, int b, int c) {
    k1 = a;
    k2 = b;
    k3 = c;
    h = a / 2 + 1;
    f1.init(a);
    f2.init(b);
    f3.init(c);
  }
  // real[k3][k2][k1] -> cplx[k3][k2][h], forward (e^{-2 pi i}), unnormalised
  void r2c(const double* in, cd* out) const {
    const int mx = std::max(k1, std::max(k2, k3));
    std::vector<cd> a(mx), b(mx);
    for (int z = 0; z < k3; ++z)
      for (int y = 0; y < k2; ++y) {
        const double* line = in + ((size_t)z * k2 + y) * k1;
        for (int x = 0; x < k1; ++x) a[x] = cd(line[x], 0.0);
        f1.exec(a.data(), 1, b.data(), -1);
        cd* o = out + ((size_t)z * k2 + y) * h;
        for (int x = 0; x < h; ++x) o[x] = b[x];
      }
    for (int z = 0; z < k3; ++z)
      for (int x = 0; x < h; ++x) {
        cd* base = out + (size_t)z * k2 * h + x;
        for (int y = 0; y < k2; ++y) a[y] = base[(size_t)y * h];
        f2.exec(a.data(), 1, b.data(), -1);
        for (int y = 0; y < k2; ++y) base[(size_t)y * h] = b[y];
      }
    for (int y = 0; y < k2; ++y)
      for (int x = 0; x < h; ++x) {
        cd* base = out + (size_t)y * h + x;
        for (int z = 0; z < k3; ++z) a[z] = base[(size_t)z * k2 * h];
        f3.exec(a.data(), 1, b.data(), -1);
        for (int z = 0; z < k3; ++z) base[(size_t)z * k2 * h] = b[z];
      }
  }
  // cplx[k3][k2][h] -> real[k3][k2][k1], backward (e^{+2 pi i}), unnormalised.
  // The input is treated as the half spectrum of a real field (imaginary parts of
  // the self-conjugate x-bins are ignored, as in any c2r transform).  `in` is clobbered.
  void c2r(cd* in, double* out) const {
    const int mx = std::max(k1, std::max(k2, k3));
    std::vector<cd> a(mx), b(mx);
    for (int y = 0; y < k2; ++y)
      for (int x = 0; x < h; ++x) {
        cd* base = in + (size_t)y * h + x;
        for (int z = 0; z < k3; ++z) a[z] = base[(size_t)z * k2 * h];
        f3.exec(a.data(), 1, b.data(), +1);
        for (int z = 0; z < k3; ++z) base[(size_t)z * k2 * h] = b[z];
      }
    for (int z = 0; z < k3; ++z)
      for (int x = 0; x < h; ++x) {
        cd* base = in + (size_t)z * k2 * h + x;
        for (int y = 0; y < k2; ++y) a[y] = base[(size_t)y * h];
        f2.exec(a.data(), 1, b.data(), +1);
        for (int y = 0; y < k2; ++y) base[(size_t)y * h] = b[y];
      }
    for (int z = 0; z < k3; ++z)
      for (int y = 0; y < k2; ++y) {
        const cd* line = in + ((size_t)z * k2 + y) * h;
        for (int x = 0; x < h; ++x) a[x] = line[x];
        for (int x = h; x < k1; ++x) a[x] = std::conj(line[k1 - x]);
        a[0] = cd(a[0].real(), 0.0);
        if (k1 % 2 == 0) a[k1 / 2] = cd(a[k1 / 2].real(), 0.0);
        f1.exec(a.data(), 1, b.data(), +1);
        double* o = out + ((size_t)z * k2 + y) * k1;
        for (int x = 0; x < k1; ++x) o[x] = b[x].real();
      }
  }
};

// ---------------------------------------------------------------------------------
// spline.F90:26-59  cardinal B-spline M_n via the alternating binomial sum
// ---------------------------------------------------------------------------------
struct Spline {
  int order = 0;
  std::vector<double> coeff;
  void init(int spline_order) {  // spline_init, spline.F90:26-44
    order = spline_order;
    coeff.assign(order + 1, 0.0);
    for (int i = 0; i <= order; ++i) {
      double factor = 1.0;
      for (int k = 1; k <= i; ++k) factor = factor * (double)k;
      for (int k = 1; k <= order - i; ++k) factor = factor * (double)k;
      factor = (double)order / factor;
      if (i % 2 == 1) factor = -factor;
      coeff[i] = factor;
    }
  }
  static double ipow(double x, int e) {  // x**e with a constant integer exponent
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
  double value(double rst) const {  // spline_value, spline.F90:47-59
    double f = 0.0;
    if ((rst > 0.0) && (rst < (double)order)) {
      const int k = (int)rst;
      for (int i = 0; i <= k; ++i) f = f + coeff[i] * ipow(rst - (double)i, order - 1);
    }
    return f;
  }
};

// ---------------------------------------------------------------------------------
// getiduv / binsearch (engproc.F90:927-1020)
// ---------------------------------------------------------------------------------
// smallest ret with coord(ret) >= v, minus one; v < coord(1) -> 0, v > coord(n) -> n
int binsearch(const double* coord, int n, double v) {
  if (v < coord[0]) return 0;
  if (v > coord[n - 1]) return n;
  int rmin = 1, rmax = n + 1;
  while (rmax - rmin > 1) {
    const int rmid = (rmin + rmax - 1) / 2;
    if (v > coord[rmid - 1])
      rmin = rmid + 1;
    else
      rmax = rmid + 1;
  }
  return rmin - 1;
}

}  // namespace

// ===================================================================================
struct orc_ctx {
  orc_params p{};
  Spline spl;
  // topology (engmain.F90:252-277)
  int nummol = 0, numatm = 0, ljtype_max = 0;
  std::vector<int> mbi;  // mol_begin_index(1:nummol+1), 1-based values
  std::vector<int> sluvid, uvspec, ljtype, numsite;
  std::vector<double> charge, ljene, ljlensq, mol_charge;
  // bins
  int numslv = 0, ermax = 0, esmax = 0;
  std::vector<int> uvmax, uvsoft, uvoff;
  std::vector<double> uvcrd, escrd;
  // accumulators (engmain.F90:283-301)
  std::vector<double> edens, ecorr, eself, slnuv, minuv, maxuv;
  double engnorm = 0, engsmpl = 0, avslf = 0, voffset = -INFTY;
  bool voffset_initialized = false;
  bool warn_bin_firsttime = true;
  // frame state
  std::vector<double> sitepos;  // (3, numatm)
  double cell[9]{}, invcl[9]{}, volume = 0, prevcl[9]{};
  double stat_weight_system = 1.0;
  std::vector<int> tagpt;  // 1-based molecule numbers of physical molecules
  int slvmax = 0;
  bool frame_ready = false;
  // reciprocal state (recpcal.F90:24-36)
  bool pme_initialized = false;
  std::vector<int> slvtag;      // per molecule (1-based mol), 1-based site offset or -1
  std::vector<double> splslv;   // (0:p-1, 3, ptrnk)
  std::vector<int> grdslv;      // (3, ptrnk)
  std::vector<double> splfc1, splfc2, splfc3, engfac;  // engfac [k3][k2][h]
  Fft3d fft;
  // realcal_self reuse (engproc.F90:716-724)
  bool usreal_valid = false;
  double usreal = 0.0;
  // intermediate-state extension (extensions/Intermediate/engproc.F90), solution mode
  bool do_intermediate = false;
  std::vector<char> zerodns_crd;          // (ermax)
  std::vector<double> edintm, uvintm;     // (ermax), (numslv)
  double soln_total = 0, soln_intm = 0, norm_intm = 0;
  // check_mol_configuration (engproc.F90:1046-1100), solution mode
  int cfg_pos = 0, cfg_str = 0;
  double cfg_lw = 0.0, cfg_up = 0.0, cfg_lwstr = 0.0, cfg_upstr = 0.0;
  std::vector<char> cfg_host;     // (nummol) molecule belongs to the host aggregate (hostspec)
  std::vector<double> cfg_mass;   // (numatm) sitemass
  std::vector<int> ref_atoms;     // refhost_specatm, 1-based atoms of the refspec molecules
  std::vector<double> refhost_crd, refhost_weight, refslt_crd, refslt_weight;
  // last placement PME potential (for cross-checks)
  std::vector<double> last_cnv;
  double last_self = 0.0;

  // column-major helpers
  double& C(int i, int j) { return cell[(i - 1) + 3 * (j - 1)]; }
  double& IC(int i, int j) { return invcl[(i - 1) + 3 * (j - 1)]; }
  double pos(int comp, int atom) const { return sitepos[(size_t)(atom - 1) * 3 + (comp - 1)]; }
};

namespace {

// --- engproc.F90:898-919 get_inverted_cell ---------------------------------------
void get_inverted_cell(orc_ctx* c) {
  auto& cl = *c;
  double v = cl.C(1, 1) * cl.C(2, 2) * cl.C(3, 3) + cl.C(1, 2) * cl.C(2, 3) * cl.C(3, 1) +
             cl.C(1, 3) * cl.C(2, 1) * cl.C(3, 2) - cl.C(1, 3) * cl.C(2, 2) * cl.C(3, 1) -
             cl.C(1, 2) * cl.C(2, 1) * cl.C(3, 3) - cl.C(1, 1) * cl.C(2, 3) * cl.C(3, 2);
  cl.volume = v;
  cl.IC(1, 1) = cl.C(2, 2) * cl.C(3, 3) - cl.C(2, 3) * cl.C(3, 2);
  cl.IC(1, 2) = cl.C(1, 3) * cl.C(3, 2) - cl.C(1, 2) * cl.C(3, 3);
  cl.IC(1, 3) = cl.C(1, 2) * cl.C(2, 3) - cl.C(1, 3) * cl.C(2, 2);
  cl.IC(2, 1) = cl.C(2, 3) * cl.C(3, 1) - cl.C(2, 1) * cl.C(3, 3);
  cl.IC(2, 2) = cl.C(1, 1) * cl.C(3, 3) - cl.C(1, 3) * cl.C(3, 1);
  cl.IC(2, 3) = cl.C(1, 3) * cl.C(2, 1) - cl.C(1, 1) * cl.C(2, 3);
  cl.IC(3, 1) = cl.C(2, 1) * cl.C(3, 2) - cl.C(2, 2) * cl.C(3, 1);
  cl.IC(3, 2) = cl.C(1, 2) * cl.C(3, 1) - cl.C(1, 1) * cl.C(3, 2);
  cl.IC(3, 3) = cl.C(1, 1) * cl.C(2, 2) - cl.C(1, 2) * cl.C(2, 1);
  for (int i = 0; i < 9; ++i) cl.invcl[i] = cl.invcl[i] / v;
}

// --- recpcal.F90:87-109 init_spline_axis ------------------------------------------
void init_spline_axis(const orc_ctx* c, int kmax, std::vector<double>& splfc) {
  splfc.assign(kmax, 0.0);
  for (int rci = 0; rci < kmax; ++rci) {
    cd rcpi(0.0, 0.0);
    for (int spi = 0; spi <= c->p.splodr - 2; ++spi) {
      const double chr = c->spl.value((double)(spi + 1));
      const double rtp2 = 2.0 * PI * (double)(spi * rci) / (double)kmax;
      rcpi += cd(chr * std::cos(rtp2), chr * std::sin(rtp2));
    }
    splfc[rci] = (rcpi * std::conj(rcpi)).real();
  }
}

// --- recpcal.F90:111-152 recpcal_spline_greenfunc ------------------------------------
void spline_greenfunc(orc_ctx* c) {
  const int K[3] = {c->p.ms1max, c->p.ms2max, c->p.ms3max};
  const int h = K[0] / 2 + 1;
  c->engfac.assign((size_t)h * K[1] * K[2], 0.0);
  const double scr = c->p.screen;
  for (int rc3 = 0; rc3 < K[2]; ++rc3)
    for (int rc2 = 0; rc2 < K[1]; ++rc2)
      for (int rc1 = 0; rc1 < h; ++rc1) {
        double factor = 0.0;
        if (rc1 == 0 && rc2 == 0 && rc3 == 0) continue;
        const int rc[3] = {rc1, rc2, rc3};
        double inm[3];
        bool zero = false;
        for (int m = 0; m < 3; ++m) {
          const int rci = rc[m], rcimax = K[m];
          if ((c->p.splodr % 2 == 1) && (2 * std::abs(rci) == rcimax)) {
            zero = true;
            break;
          }
          inm[m] = (rci <= rcimax / 2) ? (double)rci : (double)(rci - rcimax);
        }
        if (!zero) {
          double xst[3];
          for (int m = 0; m < 3; ++m)  // dot_product(invcl(:, m), inm(:))
            xst[m] = c->invcl[0 + 3 * m] * inm[0] + c->invcl[1 + 3 * m] * inm[1] + c->invcl[2 + 3 * m] * inm[2];
          double rtp2 = xst[0] * xst[0] + xst[1] * xst[1] + xst[2] * xst[2];
          const double chr = (PI * PI) * rtp2 / (scr * scr);
          factor = std::exp(-chr) / rtp2 / PI / c->volume;
          rtp2 = c->splfc1[rc1] * c->splfc2[rc2] * c->splfc3[rc3];
          factor = factor / rtp2;
        }
        c->engfac[((size_t)rc3 * K[1] + rc2) * h + rc1] = factor;
      }
  c->engfac[0] = 0.0;
}

// --- recpcal.F90:169-201 calc_gfb_pppm / gf_denom, :205-319 recpcal_pppm_greenfunc ---
void pppm_greenfunc(orc_ctx* c) {
  const int K[3] = {c->p.ms1max, c->p.ms2max, c->p.ms3max};
  const int p = c->p.splodr;
  const int h = K[0] / 2 + 1;
  std::vector<double> gf(p + 2, 0.0);  // gf_b(1:p)
  gf[1] = 1.0;
  for (int m = 1; m <= p - 1; ++m) {
    int l;
    for (l = m; l >= 1; --l)
      gf[l + 1] = 4.0 * (gf[l + 1] * (l - m) * (l - m - 0.5) - gf[l] * (double)((l - m - 1) * (l - m - 1)));
    gf[1] = 4.0 * (gf[1] * (l - m) * (l - m - 0.5));  // l = 0 after the loop
  }
  double fact = 1.0;
  for (int i = 1; i <= 2 * p - 1; ++i) fact *= i;
  for (int m = 1; m <= p; ++m) gf[m] = gf[m] / fact;
  auto denom = [&](double x, double y, double z) {
    double s[3] = {0, 0, 0};
    for (int l = p; l >= 1; --l) {
      s[0] = gf[l] + s[0] * x;
      s[1] = gf[l] + s[1] * y;
      s[2] = gf[l] + s[2] * z;
    }
    const double pr = s[0] * s[1] * s[2];
    return pr * pr;
  };
  const double eps_hoc = 0.0000001;
  double m_max[3];
  for (int a = 0; a < 3; ++a) m_max[a] = c->p.screen / (PI * K[a]) * std::pow(-std::log(eps_hoc), 0.25);
  int mm[3];
  for (int j = 0; j < 3; ++j)
    mm[j] = (int)(c->cell[3 * j] * m_max[0] + c->cell[3 * j + 1] * m_max[1] + c->cell[3 * j + 2] * m_max[2]);
  c->engfac.assign((size_t)h * K[1] * K[2], 0.0);
  for (int rc3 = 0; rc3 < K[2]; ++rc3)
    for (int rc2 = 0; rc2 < K[1]; ++rc2)
      for (int rc1 = 0; rc1 < h; ++rc1) {
        if (rc1 == 0 && rc2 == 0 && rc3 == 0) continue;
        const int rc[3] = {rc1, rc2, rc3};
        double inm[3], s2[3], k[3];
        for (int a = 0; a < 3; ++a) {
          inm[a] = (rc[a] <= K[a] / 2) ? rc[a] : rc[a] - K[a];
          const double sn = std::sin(PI * inm[a] / K[a]);
          s2[a] = sn * sn;
        }
        for (int a = 0; a < 3; ++a)
          k[a] = 2 * PI * (c->invcl[0 + 3 * a] * inm[0] + c->invcl[1 + 3 * a] * inm[1] + c->invcl[2 + 3 * a] * inm[2]);
        const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        double factor = 0.0;
        if (k2 > 0.0) {
          double sum = 0.0;
          for (int mx = -mm[0]; mx <= mm[0]; ++mx) {
            double t = PI * (inm[0] / K[0] + mx);
            const double u1 = (t == 0.0) ? 1.0 : std::pow(std::sin(t) / t, 2 * p);
            for (int my = -mm[1]; my <= mm[1]; ++my) {
              t = PI * (inm[1] / K[1] + my);
              const double u2 = (t == 0.0) ? 1.0 : std::pow(std::sin(t) / t, 2 * p);
              for (int mz = -mm[2]; mz <= mm[2]; ++mz) {
                t = PI * (inm[2] / K[2] + mz);
                const double u3 = (t == 0.0) ? 1.0 : std::pow(std::sin(t) / t, 2 * p);
                const double mN[3] = {(double)mx * K[0], (double)my * K[1], (double)mz * K[1]};  // as written
                double km[3], gam = 1.0;
                for (int a = 0; a < 3; ++a) {
                  km[a] = k[a] + 2 * PI * (c->invcl[0 + 3 * a] * mN[0] + c->invcl[1 + 3 * a] * mN[1] +
                                           c->invcl[2 + 3 * a] * mN[2]);
                  gam *= std::exp(-0.25 * (km[a] / c->p.screen) * (km[a] / c->p.screen));
                }
                sum += (k[0] * km[0] + k[1] * km[1] + k[2] * km[2]) * gam * (u1 * u2 * u3) /
                       (km[0] * km[0] + km[1] * km[1] + km[2] * km[2]);
              }
            }
          }
          factor = sum * 4.0 * PI / (k2 * denom(s2[0], s2[1], s2[2])) / c->volume;
        }
        c->engfac[((size_t)rc3 * K[1] + rc2) * h + rc1] = factor;
      }
  c->engfac[0] = 0.0;
}

// --- recpcal.F90:408-442 calc_spline_molecule -------------------------------------
void calc_spline_sites(const orc_ctx* c, const double* xyz /*(3,n)*/, int n, double* store_spline,
                       int* store_grid) {
  const int p = c->p.splodr;
  const int K[3] = {c->p.ms1max, c->p.ms2max, c->p.ms3max};
  for (int sid = 0; sid < n; ++sid) {
    const double* xst = xyz + 3 * sid;
    double inm[3];
    for (int k = 0; k < 3; ++k) {  // dot_product(invcl(k,:), xst(:))
      double factor = c->invcl[k + 0] * xst[0] + c->invcl[k + 3] * xst[1] + c->invcl[k + 6] * xst[2];
      factor = factor - std::floor(factor);
      inm[k] = factor;
    }
    for (int m = 0; m < 3; ++m) {
      const double factor = inm[m] * (double)K[m];
      const int rci = (int)factor;
      for (int spi = 0; spi < p; ++spi) {
        const double rtp2 = factor - (double)(rci - spi);
        store_spline[(size_t)sid * 3 * p + m * p + spi] = c->spl.value(rtp2);
      }
      store_grid[3 * sid + m] = rci;
    }
  }
}

inline int modulo(int a, int b) {
  int r = a % b;
  return r < 0 ? r + b : r;
}

// --- setconf.F90 / realcal.F90:888-904 calc_gmx_switching_force_params ---------------
void gmx_force_params(int pw, double lw, double up, double& A, double& B, double& Cc) {
  const double df = up - lw;
  A = -(double)pw * ((double)(pw + 4) * up - (double)(pw + 1) * lw) / (std::pow(up, pw + 2) * (df * df)) / 3.0;
  B = (double)pw * ((double)(pw + 3) * up - (double)(pw + 1) * lw) / (std::pow(up, pw + 2) * (df * df * df)) / 4.0;
  Cc = 1.0 / std::pow(up, pw) - A * (df * df * df) - B * (df * df * df * df);
}

struct LjConsts {
  double lw2, up2, lw3, up3, lw6, up6, repA, repB, repC, attA, attB, attC, ele2;
};
LjConsts lj_consts(const orc_params& p) {
  LjConsts k{};
  k.lw2 = p.lwljcut * p.lwljcut;
  k.up2 = p.upljcut * p.upljcut;
  k.lw3 = p.lwljcut * p.lwljcut * p.lwljcut;
  k.up3 = p.upljcut * p.upljcut * p.upljcut;
  k.lw6 = k.lw3 * k.lw3;
  k.up6 = k.up3 * k.up3;
  gmx_force_params(12, p.lwljcut, p.upljcut, k.repA, k.repB, k.repC);
  gmx_force_params(6, p.lwljcut, p.upljcut, k.attA, k.attB, k.attC);
  k.ele2 = p.elecut * p.elecut;
  return k;
}
inline double cube(double x) { return x * x * x; }

// LJ term inside lwljcut (realcal.F90:686-707)
inline double lj_low(const orc_params& p, const LjConsts& k, double ljeps, double ljsgm2, double dist) {
  const double invr2 = ljsgm2 / dist;
  const double invr6 = invr2 * invr2 * invr2;
  switch (p.ljswitch) {
    case 0:
    case 1:
      return 4.0 * ljeps * invr6 * (invr6 - 1.0);
    case 2: {
      const double s6 = ljsgm2 * ljsgm2 * ljsgm2;
      const double vdwa = invr6 * invr6 - s6 * s6 / (k.lw6 * k.up6);
      const double vdwb = invr6 - s6 / (k.lw3 * k.up3);
      return 4.0 * ljeps * (vdwa - vdwb);
    }
    default: {
      const double s6 = ljsgm2 * ljsgm2 * ljsgm2;
      const double vdwa = invr6 * invr6 - s6 * s6 * k.repC;
      const double vdwb = invr6 - s6 * k.attC;
      return 4.0 * ljeps * (vdwa - vdwb);
    }
  }
}
// LJ term in the switching region (realcal.F90:714-770)
inline double lj_switch(const orc_params& p, const LjConsts& k, double ljeps, double ljsgm2, double dist) {
  const double invr2 = ljsgm2 / dist;
  const double invr6 = invr2 * invr2 * invr2;
  switch (p.ljswitch) {
    case 0: {
      const double dd = dist - k.up2, den = k.up2 - k.lw2;
      return 4.0 * ljeps * invr6 * (invr6 - 1.0) * (2.0 * dist + k.up2 - 3.0 * k.lw2) * (dd * dd) / (den * den * den);
    }
    case 1: {
      const double swfac = (std::sqrt(dist) - p.lwljcut) / (p.upljcut - p.lwljcut);
      const double s3 = cube(swfac), s4 = s3 * swfac, s5 = s4 * swfac;
      return 4.0 * ljeps * invr6 * (invr6 - 1.0) * (1.0 - 10.0 * s3 + 15.0 * s4 - 6.0 * s5);
    }
    case 2: {
      const double invr3 = std::sqrt(invr6);
      const double s6 = ljsgm2 * ljsgm2 * ljsgm2;
      const double s3 = std::sqrt(s6);
      const double a = invr6 - s6 / k.up6, b = invr3 - s3 / k.up3;
      const double vdwa = k.up6 / (k.up6 - k.lw6) * (a * a);
      const double vdwb = k.up3 / (k.up3 - k.lw3) * (b * b);
      return 4.0 * ljeps * (vdwa - vdwb);
    }
    default: {
      const double s6 = ljsgm2 * ljsgm2 * ljsgm2;
      const double swfac = std::sqrt(dist) - p.lwljcut;
      const double f3 = cube(swfac), f4 = f3 * swfac;
      const double vdwa = invr6 * invr6 - s6 * s6 * (k.repA * f3 + k.repB * f4 + k.repC);
      const double vdwb = invr6 - s6 * (k.attA * f3 + k.attB * f4 + k.attC);
      return 4.0 * ljeps * (vdwa - vdwb);
    }
  }
}

// ---------------------------------------------------------------------------------
// realcal.F90: per-placement real-space machinery (cell lists rebuilt per placement)
// ---------------------------------------------------------------------------------
struct RealWork {
  // normalised (wrapped) coordinates, realcal_prepare/normalize_periodic
  std::vector<double> sitepos_normal;  // (3, numatm)
  double cell_len[3]{}, invlen[3]{};
  int bs[3]{};
  std::vector<int> nb_y, nb_z, nb_xlen;
  // solute / solvent sorted data
  std::vector<int> blk_u, belong_u, atom_u, counts_u, psum_u;
  std::vector<int> blk_v, belong_v, atom_v, counts_v, psum_v;
  std::vector<double> pos_v;  // (3, nsolv+1)
  // phase-1 lists
  std::vector<double> eps_low, sg_low, d_low, eps_sw, sg_sw, d_sw, q_el, d_el, e_t;
  std::vector<int> b_low, b_sw, b_el;
  // PME scratch
  std::vector<double> cnv;
  std::vector<cd> rcp;
};

// realcal_prepare + normalize_periodic (realcal.F90:137-146, 789-885), cuboid cells;
// a non-periodic system keeps its coordinates as they are (realcal.F90:145)
void realcal_prepare(const orc_ctx* c, const double* sitepos, RealWork& w) {
  const int n = c->numatm;
  w.sitepos_normal.assign(sitepos, sitepos + 3 * (size_t)n);
  if (c->p.boxshp == 0) return;
  for (int i = 0; i < 3; ++i) {
    w.cell_len[i] = std::fabs(c->cell[i + 3 * i]);
    w.invlen[i] = 1.0 / w.cell_len[i];
  }
  double* s = w.sitepos_normal.data();
  for (int a = 0; a < n; ++a)
    for (int i = 0; i < 3; ++i) {
      const double x = s[3 * a + i];
      s[3 * a + i] = x - w.cell_len[i] * std::floor(w.invlen[i] * x);
    }
  // second pass (realcal.F90:878-883); the x shift reads atom 1's current x, as written there
  for (int a = 0; a < n; ++a) {
    const double fy = std::floor(w.invlen[1] * s[3 * a + 1]);
    s[3 * a + 1] = s[3 * a + 1] - w.cell_len[1] * fy;
    const double fx1 = std::floor(w.invlen[0] * s[0]);
    s[3 * a + 0] = s[3 * a + 0] - w.cell_len[0] * fx1;
  }
}

// set_block_info (realcal.F90:373-437)
void set_block_info(const orc_ctx* c, RealWork& w) {
  double unit[3];
  int bmax = 0;
  for (int i = 0; i < 3; ++i) {
    w.bs[i] = (int)std::ceil(w.cell_len[i] / c->p.block_threshold);
    bmax = std::max(bmax, w.bs[i]);
    unit[i] = w.cell_len[i] / (double)w.bs[i];
  }
  std::vector<double> grid_dist((size_t)bmax * 3), box_dist((size_t)bmax * 3);
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < w.bs[j]; ++i) grid_dist[i + bmax * j] = (double)std::min(i, modulo(-i, w.bs[j])) * unit[j];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < w.bs[j]; ++i)
      box_dist[i + bmax * j] = std::min(grid_dist[i + bmax * j],
                                        std::min(grid_dist[modulo(i - 1, w.bs[j]) + bmax * j],
                                                 grid_dist[modulo(i + 1, w.bs[j]) + bmax * j]));
  const double cut = std::max(c->p.upljcut, c->p.elecut);
  const double cut2 = cut * cut;
  w.nb_y.clear();
  w.nb_z.clear();
  w.nb_xlen.clear();
  for (int k = 0; k < w.bs[2]; ++k)
    for (int j = 0; j < w.bs[1]; ++j) {
      const double by = box_dist[j + bmax * 1], bz = box_dist[k + bmax * 2];
      const double l = by * by + bz * bz;
      if (l < cut2) {
        w.nb_y.push_back(j);
        w.nb_z.push_back(k);
        w.nb_xlen.push_back((int)std::ceil(std::sqrt(cut2 - l) / unit[0]));
      }
    }
}

// blockify (realcal.F90:439-456)
void blockify(const RealWork& w, int natom, const int* atomlist, int* blk) {
  for (int i = 0; i < natom; ++i) {
    const int a = atomlist[i];
    for (int j = 0; j < 3; ++j) {
      const int bt = (int)std::floor(w.sitepos_normal[3 * (size_t)(a - 1) + j] * w.invlen[j] * (double)w.bs[j]);
      blk[3 * i + j] = modulo(bt, w.bs[j]);
    }
  }
}

// sort_block (realcal.F90:458-525): stable counting sort; psum is 1-based
void sort_block(const RealWork& w, std::vector<int>& blk, int n, std::vector<int>& belong,
                std::vector<int>& atomno, std::vector<int>& counts, std::vector<int>& psum) {
  const int nb = w.bs[0] * w.bs[1] * w.bs[2];
  counts.assign(nb, 0);
  auto cid = [&](int i) { return blk[3 * i] + w.bs[0] * (blk[3 * i + 1] + w.bs[1] * blk[3 * i + 2]); };
  for (int i = 0; i < n; ++i) counts[cid(i)]++;
  std::vector<int> pnum(nb);
  int partial = 0;
  for (int q = 0; q < nb; ++q) {
    pnum[q] = partial;
    partial += counts[q];
  }
  std::vector<int> b2(3 * (size_t)n), be2(n), at2(n);
  for (int i = 0; i < n; ++i) {
    const int q = cid(i);
    const int pos = pnum[q]++;
    b2[3 * pos] = blk[3 * i];
    b2[3 * pos + 1] = blk[3 * i + 1];
    b2[3 * pos + 2] = blk[3 * i + 2];
    be2[pos] = belong[i];
    at2[pos] = atomno[i];
  }
  blk.swap(b2);
  belong.swap(be2);
  atomno.swap(at2);
  psum.assign(nb + 1, 0);
  partial = 0;
  for (int q = 0; q < nb; ++q) {
    psum[q] = partial + 1;
    partial += counts[q];
  }
  psum[nb] = partial + 1;
}

// get_pair_energy_block (realcal.F90:585-784) -- two phases, scatter by molecule
void pair_energy_block(const orc_ctx* c, const LjConsts& k, RealWork& w, int upos, int vb, int ve,
                       double* energy_vec) {
  const orc_params& p = c->p;
  double half[3];
  for (int i = 0; i < 3; ++i) half[i] = 0.5 * w.cell_len[i];
  int n_low = 0, n_sw = 0, n_el = 0;
  for (int ui = w.psum_u[upos]; ui <= w.psum_u[upos + 1] - 1; ++ui) {
    const int ua = w.atom_u[ui - 1];
    const int lt_u = c->ljtype[ua - 1];
    const double* cu = &w.sitepos_normal[3 * (size_t)(ua - 1)];
    for (int vi = w.psum_v[vb]; vi <= w.psum_v[ve] - 1; ++vi) {
      const int va = w.atom_v[vi - 1];
      const int bv = w.belong_v[vi - 1];
      const int lt_v = c->ljtype[va - 1];
      const double* cv = &w.pos_v[3 * (size_t)(vi - 1)];
      double d2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        double d = cv[i] - cu[i];
        d = half[i] - std::fabs(half[i] - std::fabs(d));
        d2 += d * d;
      }
      const double ljeps = c->ljene[(lt_v - 1) + (size_t)c->ljtype_max * (lt_u - 1)];
      if (ljeps > 0) {
        const double sg = c->ljlensq[(lt_v - 1) + (size_t)c->ljtype_max * (lt_u - 1)];
        if (d2 <= k.lw2) {
          w.eps_low[n_low] = ljeps;
          w.sg_low[n_low] = sg;
          w.d_low[n_low] = d2;
          w.b_low[n_low] = bv;
          ++n_low;
        } else if (d2 <= k.up2) {
          w.eps_sw[n_sw] = ljeps;
          w.sg_sw[n_sw] = sg;
          w.d_sw[n_sw] = d2;
          w.b_sw[n_sw] = bv;
          ++n_sw;
        }
      }
      if (d2 <= k.ele2) {
        w.q_el[n_el] = c->charge[ua - 1] * c->charge[va - 1];
        w.d_el[n_el] = d2;
        w.b_el[n_el] = bv;
        ++n_el;
      }
    }
  }
  for (int i = 0; i < n_low; ++i) w.e_t[i] = lj_low(p, k, w.eps_low[i], w.sg_low[i], w.d_low[i]);
  for (int i = 0; i < n_low; ++i) energy_vec[w.b_low[i] - 1] += w.e_t[i];
  for (int i = 0; i < n_sw; ++i) w.e_t[i] = lj_switch(p, k, w.eps_sw[i], w.sg_sw[i], w.d_sw[i]);
  for (int i = 0; i < n_sw; ++i) energy_vec[w.b_sw[i] - 1] += w.e_t[i];
  for (int i = 0; i < n_el; ++i) {
    const double r = std::sqrt(w.d_el[i]);
    w.e_t[i] = w.q_el[i] * (1.0 - std::erf(p.screen * r)) / r;
  }
  for (int i = 0; i < n_el; ++i) energy_vec[w.b_el[i] - 1] += w.e_t[i];
}

// realcal_proc (realcal.F90:58-135) + get_pair_energy (realcal.F90:527-582)
void realcal_proc(const orc_ctx* c, int tagslt, RealWork& w, double* uvengy /*0:slvmax*/) {
  const int ns_u = c->numsite[tagslt - 1];
  int ns_v = 0;
  for (int i = 0; i < c->slvmax; ++i)
    if (c->tagpt[i] != tagslt) ns_v += c->numsite[c->tagpt[i] - 1];
  set_block_info(c, w);
  w.blk_u.assign(3 * (size_t)ns_u, 0);
  w.blk_v.assign(3 * (size_t)ns_v, 0);
  w.belong_u.assign(ns_u, tagslt);
  w.atom_u.resize(ns_u);
  for (int i = 0; i < ns_u; ++i) w.atom_u[i] = c->mbi[tagslt - 1] + i;
  w.belong_v.resize(ns_v);
  w.atom_v.resize(ns_v);
  int cnt = 0;
  for (int i = 1; i <= c->slvmax; ++i) {  // set_solv_atoms (realcal.F90:364-371)
    const int j = c->tagpt[i - 1];
    if (j == tagslt) continue;
    for (int s = 0; s < c->numsite[j - 1]; ++s) {
      w.atom_v[cnt] = c->mbi[j - 1] + s;
      w.belong_v[cnt] = i;
      ++cnt;
    }
  }
  blockify(w, ns_u, w.atom_u.data(), w.blk_u.data());
  blockify(w, ns_v, w.atom_v.data(), w.blk_v.data());
  sort_block(w, w.blk_u, ns_u, w.belong_u, w.atom_u, w.counts_u, w.psum_u);
  sort_block(w, w.blk_v, ns_v, w.belong_v, w.atom_v, w.counts_v, w.psum_v);
  w.pos_v.assign(3 * (size_t)(ns_v + 1), 0.0);
  for (int i = 0; i < ns_v; ++i)
    for (int d = 0; d < 3; ++d) w.pos_v[3 * (size_t)i + d] = w.sitepos_normal[3 * (size_t)(w.atom_v[i] - 1) + d];
  int max_u = 0;
  for (int v : w.counts_u) max_u = std::max(max_u, v);
  int max_v = 0;
  for (int y = 0; y < w.bs[1]; ++y)
    for (int z = 0; z < w.bs[2]; ++z) {
      int s = 0;
      for (int x = 0; x < w.bs[0]; ++x) s += w.counts_v[x + w.bs[0] * (y + w.bs[1] * z)];
      max_v = std::max(max_v, s);
    }
  const size_t lsize = (size_t)std::max(1, max_u * max_v);
  for (auto* v : {&w.eps_low, &w.sg_low, &w.d_low, &w.eps_sw, &w.sg_sw, &w.d_sw, &w.q_el, &w.d_el, &w.e_t})
    if (v->size() < lsize) v->resize(lsize);
  for (auto* v : {&w.b_low, &w.b_sw, &w.b_el})
    if (v->size() < lsize) v->resize(lsize);

  std::vector<double> eng(c->slvmax, 0.0);
  const LjConsts k = lj_consts(c->p);
  const int b1 = w.bs[0], b2 = w.bs[1], b3 = w.bs[2];
  for (int u3 = 0; u3 < b3; ++u3)
    for (int u2 = 0; u2 < b2; ++u2)
      for (int u1 = 0; u1 < b1; ++u1) {
        const int upos = u1 + b1 * (u2 + b2 * u3);
        if (w.psum_u[upos + 1] == w.psum_u[upos]) continue;
        for (size_t i = 0; i < w.nb_y.size(); ++i) {
          const int vy = (u2 + w.nb_y[i]) % b2, vz = (u3 + w.nb_z[i]) % b3;
          const int vbase = b1 * (vy + b2 * vz);
          const int xlen = w.nb_xlen[i];
          if (2 * xlen + 1 >= b1) {
            pair_energy_block(c, k, w, upos, vbase, vbase + b1, eng.data());
          } else {
            const int vbeg = vbase + u1 - xlen, vend = vbase + u1 + xlen + 1, vline = vbase + b1;
            if (vbeg < vbase) {
              pair_energy_block(c, k, w, upos, vbeg + b1, vline, eng.data());
              pair_energy_block(c, k, w, upos, vbase, vend, eng.data());
            } else if (vend > vline) {
              pair_energy_block(c, k, w, upos, vbeg, vline, eng.data());
              pair_energy_block(c, k, w, upos, vbase, vend - b1, eng.data());
            } else {
              pair_energy_block(c, k, w, upos, vbeg, vend, eng.data());
            }
          }
        }
      }
  for (int i = 0; i < c->slvmax; ++i) uvengy[i + 1] = eng[i];
}

// realcal_self (realcal.F90:284-328)
double realcal_self(const orc_ctx* c, int tagslt, const RealWork& w) {
  double pairep = 0.0;
  if (c->p.elmode == 2) return pairep;  // bare Coulomb (realcal.F90:294)
  double half[3];
  for (int i = 0; i < 3; ++i) half[i] = 0.5 * w.cell_len[i];
  const int ismax = c->numsite[tagslt - 1];
  for (int is = 1; is <= ismax; ++is) {
    const int ati = c->mbi[tagslt - 1] + is - 1;
    pairep += -c->charge[ati - 1] * c->charge[ati - 1] * c->p.screen / std::sqrt(PI);
    for (int js = is + 1; js <= ismax; ++js) {
      const int atj = c->mbi[tagslt - 1] + js - 1;
      double d2 = 0.0;
      for (int i = 0; i < 3; ++i) {
        double d = w.sitepos_normal[3 * (size_t)(ati - 1) + i] - w.sitepos_normal[3 * (size_t)(atj - 1) + i];
        d = half[i] - std::fabs(half[i] - std::fabs(d));
        d2 += d * d;
      }
      const double rst = std::sqrt(d2);
      pairep += -c->charge[ati - 1] * c->charge[atj - 1] * std::erf(c->p.screen * rst) / rst;
    }
  }
  return pairep;
}

// residual_ene (engproc.F90:859-869)
inline double residual_ene(const orc_ctx* c, int i, int j) {
  if (c->p.elmode == 2) return 0.0;  // engproc.F90:865
  double epcl = PI * c->mol_charge[i - 1] * c->mol_charge[j - 1] / c->p.screen / c->p.screen / c->volume;
  if (i == j) epcl = epcl / 2.0;
  return -epcl;
}

// recpcal_prepare_solute (recpcal.F90:342-406): spread, R2C, self energy, engfac, C2R
double recpcal_prepare_solute(const orc_ctx* c, int tagslt, const double* solute_xyz, RealWork& w) {
  const int p = c->p.splodr;
  const int K1 = c->p.ms1max, K2 = c->p.ms2max, K3 = c->p.ms3max, h = K1 / 2 + 1;
  const int stmax = c->numsite[tagslt - 1];
  std::vector<double> splval((size_t)stmax * 3 * p);
  std::vector<int> grdval(3 * (size_t)stmax);
  calc_spline_sites(c, solute_xyz, stmax, splval.data(), grdval.data());
  w.cnv.assign((size_t)K1 * K2 * K3, 0.0);
  for (int sid = 0; sid < stmax; ++sid) {
    const int ati = c->mbi[tagslt - 1] + sid;
    const double chr = c->charge[ati - 1];
    const double* s1 = &splval[(size_t)sid * 3 * p];
    const double* s2 = s1 + p;
    const double* s3 = s2 + p;
    for (int cg3 = 0; cg3 < p; ++cg3)
      for (int cg2 = 0; cg2 < p; ++cg2)
        for (int cg1 = 0; cg1 < p; ++cg1) {
          const int r1 = modulo(grdval[3 * sid] - cg1, K1);
          const int r2 = modulo(grdval[3 * sid + 1] - cg2, K2);
          const int r3 = modulo(grdval[3 * sid + 2] - cg3, K3);
          const double factor = chr * s1[cg1] * s2[cg2] * s3[cg3];
          w.cnv[((size_t)r3 * K2 + r2) * K1 + r1] += factor;
        }
  }
  w.rcp.resize((size_t)h * K2 * K3);
  c->fft.r2c(w.cnv.data(), w.rcp.data());
  // self energy (recpcal.F90:385-398), column-major summation order
  const int ccemax = h - 1;
  auto plane_sum = [&](int lo, int hi) {
    double s = 0.0;
    for (int r3 = 0; r3 < K3; ++r3)
      for (int r2 = 0; r2 < K2; ++r2)
        for (int r1 = lo; r1 <= hi; ++r1) {
          const size_t idx = ((size_t)r3 * K2 + r2) * h + r1;
          const cd z = w.rcp[idx];
          s += c->engfac[idx] * (z * std::conj(z)).real();
        }
    return s;
  };
  double self;
  if (K1 % 2 == 0)
    self = plane_sum(1, ccemax - 1) + 0.5 * plane_sum(0, 0) + 0.5 * plane_sum(ccemax, ccemax);
  else
    self = plane_sum(1, ccemax) + 0.5 * plane_sum(0, 0);
  for (size_t i = 0; i < w.rcp.size(); ++i) w.rcp[i] = c->engfac[i] * w.rcp[i];
  c->fft.c2r(w.rcp.data(), w.cnv.data());
  return self;
}

// recpcal_energy (recpcal.F90:451-502) for a solvent molecule i
double recpcal_energy(const orc_ctx* c, int tagslt, int i, const std::vector<double>& cnv) {
  if (c->sluvid[tagslt - 1] == 0) return std::nan("");  // rcp_fst handled by caller
  const int p = c->p.splodr;
  const int K1 = c->p.ms1max, K2 = c->p.ms2max, K3 = c->p.ms3max;
  const int svi = c->slvtag[i - 1];
  const int stmax = c->numsite[i - 1];
  double pairep = 0.0;
  for (int sid = 1; sid <= stmax; ++sid) {
    const int ptrnk = svi + sid - 1;
    const int ati = c->mbi[i - 1] + sid - 1;
    const double chr = c->charge[ati - 1];
    const double* sp = &c->splslv[(size_t)(ptrnk - 1) * 3 * p];
    const int* gr = &c->grdslv[3 * (size_t)(ptrnk - 1)];
    for (int cg3 = 0; cg3 < p; ++cg3) {
      const double fac1 = chr * sp[2 * p + cg3];
      const int rc3 = modulo(gr[2] - cg3, K3);
      for (int cg2 = 0; cg2 < p; ++cg2) {
        const double fac2 = fac1 * sp[p + cg2];
        const int rc2 = modulo(gr[1] - cg2, K2);
        const int grid1 = gr[0];
        const double* row = &cnv[((size_t)rc3 * K2 + rc2) * K1];
        for (int cg1 = 0; cg1 < p; ++cg1) {
          const double fac3 = fac2 * sp[cg1];
          const int rc1 = (grid1 >= p - 1 && grid1 < K1) ? grid1 - cg1 : (grid1 + K1 - cg1) % K1;
          pairep = pairep + fac3 * row[rc1];
        }
      }
    }
  }
  return pairep;
}

// get_uv_energy (engproc.F90:662-756) for one placement.  Returns status.
int get_uv_energy(const orc_ctx* c, int tagslt, const double* solute_xyz, double* uvengy, RealWork& w,
                  bool parallel_inner, double usreal, double* self_out) {
  // "At this moment all coordinate in the system is determined"
  std::vector<double> pos;
  const double* sitepos = c->sitepos.data();
  const int ns = c->numsite[tagslt - 1];
  const int b = c->mbi[tagslt - 1];
  std::vector<double> sxyz(3 * (size_t)ns);
  if (solute_xyz) {
    pos = c->sitepos;
    std::memcpy(&pos[3 * (size_t)(b - 1)], solute_xyz, sizeof(double) * 3 * ns);
    sitepos = pos.data();
  }
  std::memcpy(sxyz.data(), sitepos + 3 * (size_t)(b - 1), sizeof(double) * 3 * ns);
  realcal_prepare(c, sitepos, w);
  for (int k = 0; k <= c->slvmax; ++k) uvengy[k] = 0.0;
  if (c->p.elmode == 2) {  // bare Coulomb: realcal_bare per molecule (realcal.F90:155-281)
    if (self_out) *self_out = 0.0;
    if (c->sluvid[tagslt - 1] == 0) return ORC_E_RCP_FST;
    const LjConsts k = lj_consts(c->p);
    const bool periodic = c->p.boxshp != 0;
    double half[3] = {0.0, 0.0, 0.0};
    if (periodic)
      for (int i = 0; i < 3; ++i) half[i] = 0.5 * w.cell_len[i];
    // reelcut: elecut when periodic, "infinity" (1e50) otherwise (realcal.F90:170-178)
    const double reelcut = periodic ? c->p.elecut : 1.0e50;
    const int T = c->ljtype_max;
#pragma omp parallel for schedule(dynamic, 64) if (parallel_inner)
    for (int kk = 1; kk <= c->slvmax; ++kk) {
      const int i = c->tagpt[kk - 1];
      if (i == tagslt) continue;
      double pairep = 0.0;
      for (int ati = c->mbi[tagslt - 1]; ati < c->mbi[tagslt]; ++ati)
        for (int atj = c->mbi[i - 1]; atj < c->mbi[i]; ++atj) {
          double dis2 = 0.0;
          for (int a = 0; a < 3; ++a) {
            const double x = w.sitepos_normal[3 * (size_t)(ati - 1) + a] - w.sitepos_normal[3 * (size_t)(atj - 1) + a];
            const double d = periodic ? half[a] - std::fabs(half[a] - std::fabs(x)) : x;
            dis2 += d * d;
          }
          const double rst = std::sqrt(dis2);
          const int ti = c->ljtype[ati - 1], tj = c->ljtype[atj - 1];
          const double ljeps = c->ljene[(ti - 1) + (size_t)T * (tj - 1)];
          const double ljsgm2 = c->ljlensq[(ti - 1) + (size_t)T * (tj - 1)];
          double eplj = 0.0;
          if (rst <= c->p.upljcut)
            eplj = (dis2 <= k.lw2) ? lj_low(c->p, k, ljeps, ljsgm2, dis2) : lj_switch(c->p, k, ljeps, ljsgm2, dis2);
          const double epcl = (rst >= reelcut) ? 0.0 : c->charge[ati - 1] * c->charge[atj - 1] / rst;
          pairep = pairep + eplj + epcl;
        }
      uvengy[kk] = pairep;
    }
    return ORC_OK;
  }
  const double self_recip = recpcal_prepare_solute(c, tagslt, sxyz.data(), w);
  realcal_proc(c, tagslt, w, uvengy);
  uvengy[0] = self_recip;
  double pairep = std::isnan(usreal) ? realcal_self(c, tagslt, w) : usreal;
  if (self_out) *self_out = pairep;
  const double residual = residual_ene(c, tagslt, tagslt);
  uvengy[0] = uvengy[0] + pairep + residual;
  if (c->sluvid[tagslt - 1] == 0) return ORC_E_RCP_FST;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) if (parallel_inner) reduction(| : bad)
  for (int k = 1; k <= c->slvmax; ++k) {
    const int i = c->tagpt[k - 1];
    if (i == tagslt) continue;
    if (c->slvtag[i - 1] <= 0) {
      bad |= 1;
      continue;
    }
    double e = residual_ene(c, tagslt, i);
    e = e + recpcal_energy(c, tagslt, i, w.cnv);
    uvengy[k] = uvengy[k] + e;
  }
  return bad ? ORC_E_RCP_CNS : ORC_OK;
}

// volcorrect (engproc.F90:871-887), PME branch
double volcorrect(const orc_ctx* c, double weight) {
  weight = weight * c->volume;
  double total_charge = 0.0;
  for (int i = 0; i < c->nummol; ++i)
    if (c->sluvid[i] == 0 || c->sluvid[i] == 1) total_charge += c->mol_charge[i];
  if (c->p.elmode == 2) return weight;  // the charge factor only with Ewald, PME and PPPM
  const double factor = PI * (total_charge * total_charge) / (c->p.screen * c->p.screen) / c->volume / 2.0;
  return weight * std::exp(factor / c->p.temp);
}

// getiduv (engproc.F90:960-1020); returns status, writes 1-based iduv
int getiduv(orc_ctx* c, int pti, double engval, int* iduv) {
  int idmin, idnum, idpti;
  if (pti > 0) {
    idmin = c->uvoff[pti - 1];
    idnum = c->uvmax[pti - 1];
    idpti = binsearch(&c->uvcrd[idmin], idnum, engval);
  } else if (pti == 0) {
    idmin = 0;
    idnum = c->esmax;
    idpti = binsearch(c->escrd.data(), idnum, engval);
  } else {
    return ORC_E_ENG_BUG;
  }
  if (idpti <= 0) return ORC_E_ENG_MIN;
  if (idpti > idnum) return ORC_E_ENG_BUG;
  if (c->p.slttype == 1 && pti > 0 && idpti > c->uvsoft[pti - 1]) return ORC_E_ENG_SFT;
  if (idpti == idnum && engval < 1.0e3 && c->warn_bin_firsttime) {
    c->warn_bin_firsttime = false;
    if (!c->p.force_calculation) return ORC_W_MBIN;
  }
  *iduv = idmin + idpti;
  return ORC_OK;
}

// update_histogram (engproc.F90:758-856)
int update_histogram(orc_ctx* c, int tagslt, double stat_weight_solute, const double* uvengy, double* flceng) {
  double engnmfc;
  if (c->p.wgtslf == 0) {
    engnmfc = 1.0;
  } else {
    if (!c->voffset_initialized) {
      c->voffset = uvengy[0];
      c->voffset_initialized = true;
    }
    const double factor = uvengy[0] - c->voffset;
    engnmfc = (c->p.slttype == 1) ? std::exp(factor / c->p.temp) : std::exp(-factor / c->p.temp);
  }
  double total_weight = c->stat_weight_system * stat_weight_solute;
  if (c->p.estype == 2) total_weight = volcorrect(c, total_weight);
  engnmfc = engnmfc * total_weight;
  c->engnorm += engnmfc;
  c->engsmpl += 1.0;
  c->avslf += total_weight;
  int st;
  if (c->p.selfcal) {
    int iduv = 0;
    if ((st = getiduv(c, 0, uvengy[0], &iduv)) != ORC_OK) return st;
    c->eself[iduv - 1] += engnmfc;
  }
  c->minuv[0] = std::min(c->minuv[0], uvengy[0]);
  c->maxuv[0] = std::max(c->maxuv[0], uvengy[0]);
  std::vector<int> insdst(c->ermax, 0);
  for (int s = 0; s < c->numslv; ++s) flceng[s] = 0.0;
  for (int k = 1; k <= c->slvmax; ++k) {
    const int i = c->tagpt[k - 1];
    if (i == tagslt) continue;
    const int pti = c->uvspec[i - 1];
    if (pti <= 0) return ORC_E_ENG_CNS;
    const double pairep = uvengy[k];
    int iduv = 0;
    if ((st = getiduv(c, pti, pairep, &iduv)) != ORC_OK) return st;
    insdst[iduv - 1] += 1;
    flceng[pti - 1] += pairep;
    c->minuv[pti] = std::min(c->minuv[pti], pairep);
    c->maxuv[pti] = std::max(c->maxuv[pti], pairep);
  }
  if (c->p.slttype == 1)
    for (int s = 0; s < c->numslv; ++s) c->slnuv[s] += flceng[s] * engnmfc;
  for (int iduv = 0; iduv < c->ermax; ++iduv) {
    const int kk = insdst[iduv];
    if (kk == 0) continue;
    c->edens[iduv] += engnmfc * (double)kk;
  }
  if (c->p.corrcal) {
    const size_t E = (size_t)c->ermax;
    for (int iduv = 0; iduv < c->ermax; ++iduv) {
      const int kk = insdst[iduv];
      if (kk == 0) continue;
      for (int iduvp = 0; iduvp < c->ermax; ++iduvp) {
        const int q = insdst[iduvp];
        if (q == 0) continue;
        c->ecorr[iduvp + E * iduv] += engnmfc * (double)kk * (double)q;
      }
    }
  }
  if (c->do_intermediate) {  // the extension's update_histogram hunk (diff lines 198-211)
    c->soln_total = c->soln_total + engnmfc;
    bool outside = false;
    for (int iduv = 0; iduv < c->ermax; ++iduv)
      if (insdst[iduv] > 0 && c->zerodns_crd[iduv]) outside = true;
    if (!outside) {
      c->soln_intm = c->soln_intm + engnmfc;
      c->norm_intm = c->norm_intm + engnmfc;
      for (int iduv = 0; iduv < c->ermax; ++iduv) {
        const int kk = insdst[iduv];
        if (kk > 0) c->edintm[iduv] = c->edintm[iduv] + engnmfc * (double)kk;
      }
      for (int s = 0; s < c->numslv; ++s) c->uvintm[s] = c->uvintm[s] + flceng[s] * engnmfc;
    }
  }
  return ORC_OK;
}

}  // namespace

// ===================================================================================
// C ABI
// ===================================================================================
extern "C" {

double orc_spline_value(int order, double x) {
  Spline s;
  s.init(order);
  return s.value(x);
}

double orc_getscrn(double ewtoler, double elecut, int dis) {  // setconf.F90:515-535
  const double error = 1.0e-20;
  double factor = error + 1.0, ewasml = 0.0, ewalrg = 1.0e3, scrfac = 0.0;
  while (factor > error) {
    scrfac = (ewasml + ewalrg) / 2.0;
    factor = std::erfc(scrfac * elecut);
    if (dis) factor = factor / elecut;
    if (factor > ewtoler)
      ewasml = scrfac;
    else
      ewalrg = scrfac;
    factor = std::fabs(factor - ewtoler);
  }
  return scrfac;
}

int orc_enginit_species(const double* hist, int pecore, int large, double* ercrd_out, int* pemax_out,
                        int* pesoft_out) {
  // engproc.F90:163-218 for one species; ercrd is indexed 1..large
  double ecdmin = hist[0], ecfmns = hist[1], ecdcen = hist[2], eccore = hist[3], ecdmax = hist[4];
  const double eclbin = hist[5], ecfbin = hist[6], ec0bin = hist[7], finfac = hist[8];
  const int rglmax = 5;
  std::vector<double> ercrd(large + 2, 0.0);
  const double ectmvl = finfac * ecfbin;
  ecdmin = ecdmin - ectmvl;
  ecfmns = ecfmns - ectmvl;
  const double ecmns0 = ecdcen - ectmvl;
  const double ecpls0 = 2.0 * ecdcen - ecmns0;
  const double ecfpls = 2.0 * ecdcen - ecfmns;
  eccore = eccore + ecfpls - ecdcen;
  const double cdrgvl[7] = {ecdmin, ecfmns, ecmns0, ecpls0, ecfpls, eccore, ecdmax};
  int uprgcd[7];
  uprgcd[0] = 1;
  double factor = 0.0;
  for (int regn = 1; regn <= rglmax; ++regn) {
    if (regn == 1 || regn == 5) factor = eclbin;
    if (regn == 2 || regn == 4) factor = ecfbin;
    if (regn == 3) factor = ec0bin;
    const double incre = cdrgvl[regn] - cdrgvl[regn - 1];
    if (incre < factor) return ORC_E_PARAM;  // eng_ecd
    const int iduv = (int)std::lround(incre / factor);  // nint
    uprgcd[regn] = uprgcd[regn - 1] + iduv;
  }
  const int pesoft = uprgcd[rglmax] - uprgcd[0];
  const int pemax = pesoft + pecore;
  uprgcd[rglmax + 1] = pemax;
  if (pemax > large) return ORC_E_PARAM;  // eng_siz
  for (int r = 0; r <= rglmax + 1; ++r) ercrd[uprgcd[r]] = cdrgvl[r];
  const int nreg = (pecore == 0) ? rglmax : rglmax + 1;
  for (int regn = 1; regn <= nreg; ++regn) {
    const int minrg = uprgcd[regn - 1], maxrg = uprgcd[regn];
    double incre = 0.0;
    if (regn <= rglmax) incre = ercrd[maxrg] - ercrd[minrg];
    if (regn == rglmax + 1) incre = std::log(ercrd[maxrg] / ercrd[minrg]);
    factor = incre / (double)(maxrg - minrg);
    for (int iduv = minrg; iduv <= maxrg - 1; ++iduv) {
      incre = factor * (double)(iduv - minrg);
      if (regn <= rglmax) ercrd[iduv] = ercrd[minrg] + incre;
      if (regn == rglmax + 1) ercrd[iduv] = ercrd[minrg] * std::exp(incre);
    }
  }
  for (int i = 1; i <= pemax; ++i) ercrd_out[i - 1] = ercrd[i];
  *pemax_out = pemax;
  *pesoft_out = pesoft;
  return ORC_OK;
}

int orc_fft_r2c_3d(int k1, int k2, int k3, const double* in, double* out) {
  Fft3d f;
  f.init(k1, k2, k3);
  f.r2c(in, reinterpret_cast<cd*>(out));
  return ORC_OK;
}
int orc_fft_c2r_3d(int k1, int k2, int k3, const double* in, double* out) {
  Fft3d f;
  f.init(k1, k2, k3);
  std::vector<cd> tmp(reinterpret_cast<const cd*>(in), reinterpret_cast<const cd*>(in) + (size_t)(k1 / 2 + 1) * k2 * k3);
  f.c2r(tmp.data(), out);
  return ORC_OK;
}

double orc_pair_energy(const orc_params* p, double ljeps, double ljsgm2, double qq, double dist2) {
  const LjConsts k = lj_consts(*p);
  double e = 0.0;
  if (ljeps > 0) {
    if (dist2 <= k.lw2)
      e += lj_low(*p, k, ljeps, ljsgm2, dist2);
    else if (dist2 <= k.up2)
      e += lj_switch(*p, k, ljeps, ljsgm2, dist2);
  }
  if (dist2 <= k.ele2) {
    const double r = std::sqrt(dist2);
    e += qq * (1.0 - std::erf(p->screen * r)) / r;
  }
  return e;
}

int orc_create(const orc_params* p, orc_ctx** out) {
  if (!p || !out) return ORC_E_PARAM;
  if (p->splodr < 2 || p->ms1max < 2 || p->ms2max < 2 || p->ms3max < 2) return ORC_E_PARAM;
  if (p->ljswitch < 0 || p->ljswitch > 3 || p->slttype < 1 || p->slttype > 3) return ORC_E_PARAM;
  if (p->boxshp != 0 && p->boxshp != 1) return ORC_E_PARAM;
  // setconf.F90:368-372: a non-periodic system needs NVT and bare Coulomb
  if (p->boxshp == 0 && (p->estype == 2 || p->elmode != 2)) return ORC_E_SET_PRS;
  auto* c = new orc_ctx();
  c->p = *p;
  c->spl.init(p->splodr);
  c->fft.init(p->ms1max, p->ms2max, p->ms3max);
  *out = c;
  return ORC_OK;
}

void orc_destroy(orc_ctx* c) { delete c; }

int orc_set_topology(orc_ctx* c, int nummol, int numatm, const int* mbi, const int* sluvid, const int* uvspec,
                     const double* charge, const int* ljtype, int ljtype_max, const double* ljene,
                     const double* ljlensq) {
  if (!c || nummol <= 0 || numatm <= 0) return ORC_E_PARAM;
  c->nummol = nummol;
  c->numatm = numatm;
  c->mbi.assign(mbi, mbi + nummol + 1);
  c->sluvid.assign(sluvid, sluvid + nummol);
  c->uvspec.assign(uvspec, uvspec + nummol);
  c->charge.assign(charge, charge + numatm);
  c->ljtype.assign(ljtype, ljtype + numatm);
  c->ljtype_max = ljtype_max;
  c->ljene.assign(ljene, ljene + (size_t)ljtype_max * ljtype_max);
  c->ljlensq.assign(ljlensq, ljlensq + (size_t)ljtype_max * ljtype_max);
  c->numsite.resize(nummol);
  c->mol_charge.assign(nummol, 0.0);
  for (int i = 0; i < nummol; ++i) {
    c->numsite[i] = mbi[i + 1] - mbi[i];
    if (c->numsite[i] <= 0) return ORC_E_PARAM;
    double s = 0.0;  // setconf.F90:832-834
    for (int a = mbi[i]; a < mbi[i + 1]; ++a) s += charge[a - 1];
    c->mol_charge[i] = s;
  }
  if (mbi[nummol] - 1 != numatm) return ORC_E_PARAM;
  // tagpt (engproc.F90:336-348)
  c->tagpt.clear();
  for (int i = 1; i <= nummol; ++i)
    if (sluvid[i - 1] == 0 || sluvid[i - 1] == 1) c->tagpt.push_back(i);
  c->slvmax = (int)c->tagpt.size();
  c->pme_initialized = false;
  c->usreal_valid = false;
  return ORC_OK;
}

int orc_set_bins(orc_ctx* c, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd, int esmax,
                 const double* escrd) {
  if (!c || numslv <= 0) return ORC_E_PARAM;
  c->numslv = numslv;
  c->uvmax.assign(uvmax, uvmax + numslv);
  c->uvsoft.assign(uvsoft, uvsoft + numslv);
  c->uvoff.assign(numslv, 0);
  int e = 0;
  for (int s = 0; s < numslv; ++s) {
    c->uvoff[s] = e;
    e += uvmax[s];
  }
  c->ermax = e;
  c->uvcrd.assign(uvcrd, uvcrd + e);
  c->esmax = esmax;
  c->escrd.assign(escrd, escrd + std::max(esmax, 0));
  c->edens.assign(e, 0.0);
  if (c->p.corrcal) c->ecorr.assign((size_t)e * e, 0.0);
  c->eself.assign(std::max(esmax, 0), 0.0);
  c->slnuv.assign(numslv, 0.0);
  c->minuv.assign(numslv + 1, INFTY);
  c->maxuv.assign(numslv + 1, -INFTY);
  c->voffset = -INFTY;
  return orc_clear(c);
}

int orc_clear(orc_ctx* c) {  // engclear, engproc.F90:276-288
  std::fill(c->edens.begin(), c->edens.end(), 0.0);
  std::fill(c->ecorr.begin(), c->ecorr.end(), 0.0);
  if (c->do_intermediate) {  // engclear hunk of the intermediate-state extension
    std::fill(c->edintm.begin(), c->edintm.end(), 0.0);
    std::fill(c->uvintm.begin(), c->uvintm.end(), 0.0);
    c->norm_intm = 0.0;
  }
  std::fill(c->eself.begin(), c->eself.end(), 0.0);
  std::fill(c->slnuv.begin(), c->slnuv.end(), 0.0);
  c->avslf = 0.0;
  c->engnorm = 0.0;
  c->engsmpl = 0.0;
  return ORC_OK;
}

int orc_frame(orc_ctx* c, const double* sitepos, const double* cell, double stat_weight_system) {
  if (!c || c->numatm <= 0 || c->ermax <= 0) return ORC_E_PARAM;
  c->sitepos.assign(sitepos, sitepos + 3 * (size_t)c->numatm);
  std::memcpy(c->cell, cell, sizeof(double) * 9);
  if (c->p.boxshp == 0) {  // non-periodic: bare Coulomb only, no cell, no reciprocal set-up
    c->stat_weight_system = stat_weight_system;
    get_inverted_cell(c);
    c->frame_ready = true;
    return ORC_OK;
  }
  // non-cuboid cells stop the reference (realcal.F90:859-866)
  if (std::fabs(cell[3]) > 1e-8 || std::fabs(cell[6]) > 1e-8 || std::fabs(cell[7]) > 1e-8 ||
      std::fabs(cell[1]) > 1e-8 || std::fabs(cell[2]) > 1e-8 || std::fabs(cell[5]) > 1e-8 ||
      !(cell[0] > 0) || !(cell[4] > 0) || !(cell[8] > 0))
    return ORC_E_NONCUBOID;
  c->stat_weight_system = stat_weight_system;
  get_inverted_cell(c);
  if (!c->pme_initialized) {  // recpcal_init (recpcal.F90:42-85)
    c->slvtag.assign(c->nummol, -1);
    int ptrnk = 0;
    for (int k = 0; k < c->slvmax; ++k) {
      const int m = c->tagpt[k];
      c->slvtag[m - 1] = ptrnk + 1;
      ptrnk += c->numsite[m - 1];
    }
    c->splslv.assign((size_t)ptrnk * 3 * c->p.splodr, 0.0);
    c->grdslv.assign(3 * (size_t)ptrnk, 0);
    init_spline_axis(c, c->p.ms1max, c->splfc1);
    init_spline_axis(c, c->p.ms2max, c->splfc2);
    init_spline_axis(c, c->p.ms3max, c->splfc3);
  }
  bool changed = !c->pme_initialized;
  for (int i = 0; i < 9; ++i) changed = changed || (c->prevcl[i] != c->cell[i]);
  if (changed) {
    if (c->p.elmode == 1)
      pppm_greenfunc(c);
    else
      spline_greenfunc(c);
  }
  std::memcpy(c->prevcl, c->cell, sizeof(double) * 9);
  c->pme_initialized = true;
  // recpcal_prepare_solvent for every physical molecule (engproc.F90:378-382)
#pragma omp parallel for schedule(dynamic, 64)
  for (int k = 0; k < c->slvmax; ++k) {
    const int i = c->tagpt[k];
    const int svi = c->slvtag[i - 1];
    calc_spline_sites(c, &c->sitepos[3 * (size_t)(c->mbi[i - 1] - 1)], c->numsite[i - 1],
                      &c->splslv[(size_t)(svi - 1) * 3 * c->p.splodr], &c->grdslv[3 * (size_t)(svi - 1)]);
  }
  c->frame_ready = true;
  return ORC_OK;
}

int orc_slvmax(const orc_ctx* c) { return c ? c->slvmax : -1; }

int orc_set_aggregate(orc_ctx* c, const int* host_mol, const double* sitemass) {
  if (!c || c->nummol <= 0 || !host_mol || !sitemass) return ORC_E_PARAM;
  c->cfg_host.assign(c->nummol, 0);
  for (int i = 0; i < c->nummol; ++i) c->cfg_host[i] = host_mol[i] != 0;
  c->cfg_mass.assign(sitemass, sitemass + c->numatm);
  return ORC_OK;
}

int orc_set_reference_structure(orc_ctx* c, const int* ref_mol, const double* refhost_crd,
                                const double* refhost_weight, int refslt_natom, const double* refslt_crd,
                                const double* refslt_weight) {
  if (!c || c->nummol <= 0 || !ref_mol || refslt_natom <= 0) return ORC_E_PARAM;
  c->ref_atoms.clear();
  for (int i = 0; i < c->nummol; ++i)  // load_refstructure, insertion.F90:630-646
    if (ref_mol[i])
      for (int a = c->mbi[i]; a < c->mbi[i + 1]; ++a) c->ref_atoms.push_back(a);
  const size_t nh = c->ref_atoms.size();
  c->refhost_crd.assign(refhost_crd, refhost_crd + 3 * nh);
  c->refhost_weight.assign(refhost_weight, refhost_weight + nh);
  c->refslt_crd.assign(refslt_crd, refslt_crd + 3 * (size_t)refslt_natom);
  c->refslt_weight.assign(refslt_weight, refslt_weight + refslt_natom);
  return ORC_OK;
}

int orc_set_configuration_check(orc_ctx* c, int insposition, double lwreg, double upreg, int insstructure,
                                double lwstr, double upstr) {
  if (!c || c->nummol <= 0) return ORC_E_PARAM;
  c->cfg_pos = c->cfg_str = 0;
  const int pos = (insposition >= 2 && insposition <= 5) ? insposition : 0;
  if (c->p.boxshp == 0 && (pos == 3 || pos == 4)) return ORC_E_ENG_SLB;  // engproc.F90:1087
  if (pos >= 2 && pos <= 4 && c->cfg_host.empty()) return ORC_E_PARAM;
  if ((pos == 5 || insstructure == 1) && c->refslt_weight.empty()) return ORC_E_PARAM;
  c->cfg_pos = pos;
  c->cfg_str = insstructure == 1 ? 1 : 0;
  c->cfg_lw = lwreg;
  c->cfg_up = upreg;
  c->cfg_lwstr = lwstr;
  c->cfg_upstr = upstr;
  return ORC_OK;
}

namespace {

// --- bestfit.F90 ---------------------------------------------------------------------
// center_of_mass (:158-172) of n points (3, n) with weights m
int com_points(int n, const double* x, const double* m, double com[3]) {
  double msum = 0.0;
  for (int k = 0; k < n; ++k) msum += m[k];
  if (msum == 0.0) return ORC_E_PARAM;  // bst_zrw
  for (int i = 0; i < 3; ++i) {
    double dot = 0.0;
    for (int k = 0; k < n; ++k) dot += x[3 * k + i] * m[k];
    com[i] = dot / msum;
  }
  return ORC_OK;
}

// The largest eigenpair of a symmetric 4 x 4 matrix, for find_rotation_quaternion's dsyev
// call (:146-155).  LAPACK is not in the reference tree; its result is restated with the
// cyclic Jacobi method (Golub & Van Loan, Matrix Computations, section 8.5) and checked
// against numpy.linalg.eigh in the tests.
void top_eigenvector4(double a[4][4], double vec[4]) {
  double v[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < 4; ++i) {
      diag += a[i][i] * a[i][i];
      for (int j = i + 1; j < 4; ++j) off += 2.0 * a[i][j] * a[i][j];
    }
    if (off <= 1e-32 * (off + diag)) break;
    for (int p = 0; p < 4; ++p)
      for (int q = p + 1; q < 4; ++q) {
        if (a[p][q] == 0.0) continue;
        const double tau = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = std::copysign(1.0, tau) / (std::fabs(tau) + std::hypot(1.0, tau));
        const double cs = 1.0 / std::hypot(1.0, t), sn = t * cs;
        for (int k = 0; k < 4; ++k) {  // columns p, q
          const double x = a[k][p], y = a[k][q];
          a[k][p] = cs * x - sn * y;
          a[k][q] = sn * x + cs * y;
        }
        for (int k = 0; k < 4; ++k) {  // rows p, q
          const double x = a[p][k], y = a[q][k];
          a[p][k] = cs * x - sn * y;
          a[q][k] = sn * x + cs * y;
        }
        a[p][q] = a[q][p] = 0.0;
        for (int k = 0; k < 4; ++k) {
          const double x = v[k][p], y = v[k][q];
          v[k][p] = cs * x - sn * y;
          v[k][q] = sn * x + cs * y;
        }
      }
  }
  int top = 0;
  for (int i = 1; i < 4; ++i)
    if (a[i][i] > a[top][top]) top = i;
  for (int i = 0; i < 4; ++i) vec[i] = v[i][top];
}

// quaternion product (:49-65) and rotate (:75-87)
void qprod(const double a[4], const double b[4], double p[4]) {
  p[0] = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  p[1] = (a[2] * b[3] - a[3] * b[2]) + a[0] * b[1] + b[0] * a[1];
  p[2] = (a[3] * b[1] - a[1] * b[3]) + a[0] * b[2] + b[0] * a[2];
  p[3] = (a[1] * b[2] - a[2] * b[1]) + a[0] * b[3] + b[0] * a[3];
}
void qrotate(const double x[3], const double r[4], double out[3]) {
  const double q2[4] = {0.0, x[0], x[1], x[2]}, cj[4] = {r[0], -r[1], -r[2], -r[3]};
  double t[4], res[4];
  qprod(r, q2, t);
  qprod(t, cj, res);
  for (int i = 0; i < 3; ++i) out[i] = res[i + 1];
}

// fit_a_rotate_b (:215-242): fit a (3, na) onto refa with weights massa, apply to b (3, nb)
int fit_a_rotate_b(int na, const double* refa, const double* a, const double* massa, int nb, const double* b,
                   double* bout) {
  double cref[3], ca[3];
  int st = com_points(na, refa, massa, cref);
  if (st == ORC_OK) st = com_points(na, a, massa, ca);
  if (st != ORC_OK) return st;
  double ip[3][3];  // inner_prod(j, i) = sum refPt(i, :) movedPt(j, :) masses(:)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < na; ++k) s += (refa[3 * k + i] - cref[i]) * (a[3 * k + j] - ca[j]) * massa[k];
      ip[j][i] = s;
    }
  double m[4][4];  // find_rotation_quaternion (:107-156), both triangles
  m[0][0] = ip[0][0] + ip[1][1] + ip[2][2];
  m[1][1] = ip[0][0] - ip[1][1] - ip[2][2];
  m[2][2] = -ip[0][0] + ip[1][1] - ip[2][2];
  m[3][3] = -ip[0][0] - ip[1][1] + ip[2][2];
  m[0][1] = m[1][0] = ip[1][2] - ip[2][1];
  m[0][2] = m[2][0] = ip[2][0] - ip[0][2];
  m[0][3] = m[3][0] = ip[0][1] - ip[1][0];
  m[1][2] = m[2][1] = ip[0][1] + ip[1][0];
  m[2][3] = m[3][2] = ip[1][2] + ip[2][1];
  m[1][3] = m[3][1] = ip[2][0] + ip[0][2];
  double rot[4];
  top_eigenvector4(m, rot);
  for (int k = 0; k < nb; ++k) {
    const double d[3] = {b[3 * k] - ca[0], b[3 * k + 1] - ca[1], b[3 * k + 2] - ca[2]};
    double r[3];
    qrotate(d, rot, r);
    for (int i = 0; i < 3; ++i) bout[3 * k + i] = r[i] + cref[i];
  }
  return ORC_OK;
}

// rmsd_nofit (:256-270)
double rmsd_nofit(int n, const double* A, const double* B, const double* m) {
  double msum = 0.0, disp = 0.0;
  for (int k = 0; k < n; ++k) msum += m[k];
  for (int k = 0; k < n; ++k) {
    double d2 = 0.0;
    for (int i = 0; i < 3; ++i) d2 += (B[3 * k + i] - A[3 * k + i]) * (B[3 * k + i] - A[3 * k + i]);
    disp += m[k] * d2;
  }
  return std::sqrt(disp / msum);
}

// center_of_mass (bestfit.F90:158-172) of the listed atoms (1-based), in their order
int center_of_mass(const orc_ctx* c, const std::vector<int>& atoms, double com[3]) {
  double msum = 0.0;
  for (int a : atoms) msum += c->cfg_mass[a - 1];
  if (msum == 0.0) return ORC_E_PARAM;  // bst_zrw
  for (int i = 0; i < 3; ++i) {
    double dot = 0.0;
    for (int a : atoms) dot += c->pos(i + 1, a) * c->cfg_mass[a - 1];
    com[i] = dot / msum;
  }
  return ORC_OK;
}

// check_mol_configuration for solute molecule tagslt (engproc.F90:1046-1100,
// relative_com :1150-1172, com_aggregate insertion.F90:539-566).  refslt_bestfit is the
// reference solute carried into the frame (insposition 5), computed once per call.
int config_rejected(const orc_ctx* c, int tagslt, const std::vector<double>& refslt_bestfit, bool* out) {
  *out = false;
  const int b = c->mbi[tagslt - 1], n = c->numsite[tagslt - 1];
  const double* sx = &c->sitepos[3 * (size_t)(b - 1)];
  if (c->cfg_pos >= 2 && c->cfg_pos <= 4) {
    std::vector<int> slt, agg;
    for (int a = b; a < c->mbi[tagslt]; ++a) slt.push_back(a);
    for (int i = 0; i < c->nummol; ++i)
      if (c->cfg_host[i])
        for (int a = c->mbi[i]; a < c->mbi[i + 1]; ++a) agg.push_back(a);
    double scom[3], acom[3];
    int st = center_of_mass(c, slt, scom);
    if (st == ORC_OK) st = center_of_mass(c, agg, acom);
    if (st != ORC_OK) return st;
    const double dx[3] = {scom[0] - acom[0], scom[1] - acom[1], scom[2] - acom[2]};
    double distance;
    if (c->cfg_pos == 2) {
      distance = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    } else {
      const double len3 = std::sqrt(c->cell[6] * c->cell[6] + c->cell[7] * c->cell[7] + c->cell[8] * c->cell[8]);
      distance = (c->invcl[2] * dx[0] + c->invcl[5] * dx[1] + c->invcl[8] * dx[2]) * len3;
      if (c->cfg_pos == 4) distance = std::fabs(distance);
    }
    if ((c->cfg_lw > distance) || (distance > c->cfg_up)) {
      *out = true;
      return ORC_OK;
    }
  } else if (c->cfg_pos == 5) {
    if (n != (int)c->refslt_weight.size()) return ORC_E_ENG_BUG;
    const double distance = rmsd_nofit(n, refslt_bestfit.data(), sx, c->refslt_weight.data());
    if ((c->cfg_lw > distance) || (distance > c->cfg_up)) {
      *out = true;
      return ORC_OK;
    }
  }
  if (c->cfg_str == 1) {  // INSSTR_RMSD: rmsd_bestfit(refslt_crd, the solute)
    if (n != (int)c->refslt_weight.size()) return ORC_E_ENG_BUG;
    std::vector<double> fitted(3 * (size_t)n);
    const int st = fit_a_rotate_b(n, c->refslt_crd.data(), sx, c->refslt_weight.data(), n, sx, fitted.data());
    if (st != ORC_OK) return st;
    const double distance = rmsd_nofit(n, c->refslt_crd.data(), fitted.data(), c->refslt_weight.data());
    if ((c->cfg_lwstr > distance) || (distance > c->cfg_upstr)) *out = true;
  }
  return ORC_OK;
}

}  // namespace

int orc_fit_a_rotate_b(int na, const double* refa, const double* a, const double* massa, int nb, const double* b,
                       double* bout) {
  if (na <= 0 || nb < 0 || !refa || !a || !massa || (nb > 0 && (!b || !bout))) return ORC_E_PARAM;
  return fit_a_rotate_b(na, refa, a, massa, nb, b, bout);
}

int orc_placements(orc_ctx* c, int nplace, const int* tagslt, const double* solute_sitepos,
                   const double* stat_weight_solute, double* uvengy_out, double* flceng_out, int nthreads) {
  if (!c || !c->frame_ready || nplace < 0 || !tagslt) return ORC_E_PARAM;
  if (nplace == 0) return ORC_OK;
  const int S = c->slvmax + 1;
  for (int q = 0; q < nplace; ++q) {
    if (tagslt[q] < 1 || tagslt[q] > c->nummol) return ORC_E_PARAM;
    if (c->sluvid[tagslt[q] - 1] == 0) return ORC_E_RCP_FST;
  }
  const int ns0 = c->numsite[tagslt[0] - 1];
  std::vector<double> uv((size_t)nplace * S);
  // the loop's skipcond (engproc.F90:389-390): rejected solution-mode placements compute
  // and accumulate nothing
  std::vector<char> rejected(nplace, 0);
  if (c->p.slttype == 1 && (c->cfg_pos != 0 || c->cfg_str != 0)) {
    std::vector<double> bestfit;  // refslt_bestfit: the reference host fitted onto the frame's
    if (c->cfg_pos == 5) {
      const int nh = (int)c->ref_atoms.size(), nsr = (int)c->refslt_weight.size();
      std::vector<double> hostcrd(3 * (size_t)nh);
      for (int k = 0; k < nh; ++k)
        for (int i = 0; i < 3; ++i) hostcrd[3 * k + i] = c->pos(i + 1, c->ref_atoms[k]);
      bestfit.resize(3 * (size_t)nsr);
      const int st = fit_a_rotate_b(nh, hostcrd.data(), c->refhost_crd.data(), c->refhost_weight.data(), nsr,
                                    c->refslt_crd.data(), bestfit.data());
      if (st != ORC_OK) return st;
    }
    for (int q = 0; q < nplace; ++q) {
      bool r = false;
      const int st = config_rejected(c, tagslt[q], bestfit, &r);
      if (st != ORC_OK) return st;
      rejected[q] = r;
    }
  }
#ifdef _OPENMP
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  const int nt = 1;
  (void)nthreads;
#endif
  // realcal_self: REFS rigid computes it at the first placement of the run and reuses it
  // (engproc.F90:716-724); everything else recomputes it (same coordinates -> same value).
  const bool rigid = (c->p.slttype == 2);
  if (rigid && !c->usreal_valid) {
    RealWork w;
    const int b = c->mbi[tagslt[0] - 1];
    std::vector<double> pos = c->sitepos;
    if (solute_sitepos) std::memcpy(&pos[3 * (size_t)(b - 1)], solute_sitepos, sizeof(double) * 3 * ns0);
    realcal_prepare(c, pos.data(), w);
    c->usreal = realcal_self(c, tagslt[0], w);
    c->usreal_valid = true;
  }
  const double usreal = rigid ? c->usreal : std::nan("");
  int status = ORC_OK;
  const bool outer = (nplace >= nt) || nt == 1;
  if (outer) {
#pragma omp parallel num_threads(nt)
    {
      RealWork w;
#pragma omp for schedule(dynamic, 1)
      for (int q = 0; q < nplace; ++q) {
        const int ns = c->numsite[tagslt[q] - 1];
        const double* sx = solute_sitepos ? solute_sitepos + (size_t)3 * ns0 * q : nullptr;
        (void)ns;
        if (rejected[q]) continue;
        int st = get_uv_energy(c, tagslt[q], sx, &uv[(size_t)q * S], w, false, usreal, nullptr);
        if (st != ORC_OK) {
#pragma omp critical
          status = status ? status : st;
        }
        if (nplace == 1) {
#pragma omp critical
          {
            c->last_cnv = w.cnv;
            c->last_self = uv[0];
          }
        }
      }
    }
  } else {
    RealWork w;
#ifdef _OPENMP
    omp_set_num_threads(nt);
#endif
    for (int q = 0; q < nplace; ++q) {
      const double* sx = solute_sitepos ? solute_sitepos + (size_t)3 * ns0 * q : nullptr;
      if (rejected[q]) continue;
      int st = get_uv_energy(c, tagslt[q], sx, &uv[(size_t)q * S], w, true, usreal, nullptr);
      if (st != ORC_OK) status = status ? status : st;
      c->last_cnv = w.cnv;
    }
  }
  if (status != ORC_OK) return status;
  std::vector<double> fl(c->numslv);
  for (int q = 0; q < nplace; ++q) {
    if (rejected[q]) {
      if (uvengy_out) std::fill(uvengy_out + (size_t)q * S, uvengy_out + (size_t)(q + 1) * S, 0.0);
      if (flceng_out) std::fill(flceng_out + (size_t)q * c->numslv, flceng_out + (size_t)(q + 1) * c->numslv, 0.0);
      continue;
    }
    const double sw = stat_weight_solute ? stat_weight_solute[q] : 1.0;
    const int st = update_histogram(c, tagslt[q], sw, &uv[(size_t)q * S], fl.data());
    if (uvengy_out) std::memcpy(uvengy_out + (size_t)q * S, &uv[(size_t)q * S], sizeof(double) * S);
    if (flceng_out) std::memcpy(flceng_out + (size_t)q * c->numslv, fl.data(), sizeof(double) * c->numslv);
    if (st != ORC_OK) return st;
  }
  return ORC_OK;
}

int orc_get_accum(const orc_ctx* c, double* edens, double* ecorr, double* eself, double* slnuv, double* minuv,
                  double* maxuv, double* scalars) {
  if (!c) return ORC_E_PARAM;
  if (edens) std::copy(c->edens.begin(), c->edens.end(), edens);
  if (ecorr && c->p.corrcal) std::copy(c->ecorr.begin(), c->ecorr.end(), ecorr);
  if (eself) std::copy(c->eself.begin(), c->eself.end(), eself);
  if (slnuv) std::copy(c->slnuv.begin(), c->slnuv.end(), slnuv);
  if (minuv) std::copy(c->minuv.begin(), c->minuv.end(), minuv);
  if (maxuv) std::copy(c->maxuv.begin(), c->maxuv.end(), maxuv);
  if (scalars) {
    scalars[0] = c->engnorm;
    scalars[1] = c->engsmpl;
    scalars[2] = c->avslf;
    scalars[3] = c->voffset;
    scalars[4] = c->voffset_initialized ? 1.0 : 0.0;
  }
  return ORC_OK;
}

int orc_last_cnvslt(const orc_ctx* c, double* out, double* self_energy) {
  if (!c || c->last_cnv.empty()) return ORC_E_PARAM;
  if (out) std::copy(c->last_cnv.begin(), c->last_cnv.end(), out);
  if (self_energy) *self_energy = c->last_self;
  return ORC_OK;
}

int orc_recip_parts(const orc_ctx* c, int tagslt, const double* solute_sitepos, double* out, double* self_out) {
  // recpcal_prepare_solute + recpcal_energy alone (no real space, no residual)
  if (!c || !c->frame_ready) return ORC_E_PARAM;
  const int ns = c->numsite[tagslt - 1];
  const int b = c->mbi[tagslt - 1];
  std::vector<double> sx(3 * (size_t)ns);
  if (solute_sitepos)
    std::memcpy(sx.data(), solute_sitepos, sizeof(double) * 3 * ns);
  else
    std::memcpy(sx.data(), &c->sitepos[3 * (size_t)(b - 1)], sizeof(double) * 3 * ns);
  RealWork w;
  const double self = recpcal_prepare_solute(c, tagslt, sx.data(), w);
  for (int k = 0; k < c->slvmax; ++k) {
    const int i = c->tagpt[k];
    out[k] = (i == tagslt) ? 0.0 : recpcal_energy(c, tagslt, i, w.cnv);
  }
  if (self_out) *self_out = self;
  return ORC_OK;
}

// Per-molecule derivatives of uvengy(k) (get_uv_energy, engproc.F90:662-756) with
// respect to the solute's per-site parameters, FP64.  For solute site s and solvent
// molecule k (tagpt order), out[k * 3 ns + 3 s + {0, 1, 2}] holds du_k / d{q_s, eps_s,
// sigma_s}: q_s the charge as the topology holds it (e x 18.22261721), eps_s and sigma_s
// the site's LJ parameters under ljene = sqrt(eps_s eps_t) and ljlensq =
// ((sigma_s + sigma_t) / 2)^2 (cmbrule 0) or sigma_s sigma_t (cmbrule 1), setconf.F90:779-823.
//   d/dq_s:  sum_t q_t erfc(beta r)/r within elecut (realcal.F90:700-710), plus
//            sum_t q_t phi_s(r_t) with phi_s the PME potential of a unit charge on s
//            (recpcal_prepare_solute + recpcal_energy with one site), plus
//            -pi Q_k / (beta^2 V) (residual_ene, engproc.F90:859-869);
//   the LJ term of every switching form is 4 eps (vdwa - vdwb) with vdwa ~ sigma^12 and
//   vdwb ~ sigma^6 (realcal.F90:686-770), so dLJ/deps_s = LJ / (2 eps_s) and
//   dLJ/d(sigma^2) = 4 eps (6 vdwa - 3 vdwb) / sigma^2.
// The sum over pairs is a direct minimum-image loop (the cell list only selects pairs
// within the cutoffs).  eps_s = 0 or sigma_s = 0 report 0 for that parameter.
}  // extern "C"
namespace {
void lj_parts(const orc_params& p, const LjConsts& k, double x, double dist, double& vdwa, double& vdwb) {
  const double invr2 = x / dist;
  const double invr6 = invr2 * invr2 * invr2;
  const double s6 = x * x * x;
  if (dist <= k.lw2) {
    switch (p.ljswitch) {
      case 0:
      case 1:
        vdwa = invr6 * invr6;
        vdwb = invr6;
        return;
      case 2:
        vdwa = invr6 * invr6 - s6 * s6 / (k.lw6 * k.up6);
        vdwb = invr6 - s6 / (k.lw3 * k.up3);
        return;
      default:
        vdwa = invr6 * invr6 - s6 * s6 * k.repC;
        vdwb = invr6 - s6 * k.attC;
        return;
    }
  }
  switch (p.ljswitch) {
    case 0: {
      const double dd = dist - k.up2, den = k.up2 - k.lw2;
      const double sw = (2.0 * dist + k.up2 - 3.0 * k.lw2) * (dd * dd) / (den * den * den);
      vdwa = invr6 * invr6 * sw;
      vdwb = invr6 * sw;
      return;
    }
    case 1: {
      const double swfac = (std::sqrt(dist) - p.lwljcut) / (p.upljcut - p.lwljcut);
      const double s3 = cube(swfac), s4 = s3 * swfac, s5 = s4 * swfac;
      const double sw = 1.0 - 10.0 * s3 + 15.0 * s4 - 6.0 * s5;
      vdwa = invr6 * invr6 * sw;
      vdwb = invr6 * sw;
      return;
    }
    case 2: {
      const double invr3 = std::sqrt(invr6), s3 = std::sqrt(s6);
      const double a = invr6 - s6 / k.up6, b = invr3 - s3 / k.up3;
      vdwa = k.up6 / (k.up6 - k.lw6) * (a * a);
      vdwb = k.up3 / (k.up3 - k.lw3) * (b * b);
      return;
    }
    default: {
      const double swfac = std::sqrt(dist) - p.lwljcut;
      const double f3 = cube(swfac), f4 = f3 * swfac;
      vdwa = invr6 * invr6 - s6 * s6 * (k.repA * f3 + k.repB * f4 + k.repC);
      vdwb = invr6 - s6 * (k.attA * f3 + k.attB * f4 + k.attC);
      return;
    }
  }
}

// PME potential on the grid of a unit charge at xyz (recpcal.F90:342-406 for one site)
void unit_site_potential(const orc_ctx* c, const double* xyz, std::vector<double>& cnv) {
  const int p = c->p.splodr;
  const int K1 = c->p.ms1max, K2 = c->p.ms2max, K3 = c->p.ms3max, h = K1 / 2 + 1;
  std::vector<double> spl(3 * (size_t)p);
  int grd[3];
  calc_spline_sites(c, xyz, 1, spl.data(), grd);
  cnv.assign((size_t)K1 * K2 * K3, 0.0);
  for (int cg3 = 0; cg3 < p; ++cg3)
    for (int cg2 = 0; cg2 < p; ++cg2)
      for (int cg1 = 0; cg1 < p; ++cg1) {
        const int r1 = modulo(grd[0] - cg1, K1), r2 = modulo(grd[1] - cg2, K2), r3 = modulo(grd[2] - cg3, K3);
        cnv[((size_t)r3 * K2 + r2) * K1 + r1] += spl[cg1] * spl[p + cg2] * spl[2 * p + cg3];
      }
  std::vector<cd> rcp((size_t)h * K2 * K3);
  c->fft.r2c(cnv.data(), rcp.data());
  for (size_t i = 0; i < rcp.size(); ++i) rcp[i] = c->engfac[i] * rcp[i];
  c->fft.c2r(rcp.data(), cnv.data());
}
}  // namespace
extern "C" {

int orc_adjoint(const orc_ctx* c, int tagslt, const double* solute_sitepos, int cmbrule, double* out) {
  if (!c || !c->frame_ready || !out || tagslt < 1 || tagslt > c->nummol || cmbrule < 0 || cmbrule > 1)
    return ORC_E_PARAM;
  const int ns = c->numsite[tagslt - 1];
  const int b = c->mbi[tagslt - 1];
  const int P = 3 * ns;
  std::vector<double> sx(3 * (size_t)ns);
  if (solute_sitepos)
    std::memcpy(sx.data(), solute_sitepos, sizeof(double) * 3 * ns);
  else
    std::memcpy(sx.data(), &c->sitepos[3 * (size_t)(b - 1)], sizeof(double) * 3 * ns);
  std::fill(out, out + (size_t)c->slvmax * P, 0.0);
  const LjConsts k = lj_consts(c->p);
  const int T = c->ljtype_max;
  const double L[3] = {c->cell[0], c->cell[4], c->cell[8]};
  auto wrap = [&](double v, int a) { return v - L[a] * std::floor(v / L[a]); };
  const double resid = PI / c->p.screen / c->p.screen / c->volume;
  // reciprocal space: one unit-charge potential per solute site
  std::vector<std::vector<double>> cnv(ns);
  for (int s = 0; s < ns; ++s) unit_site_potential(c, &sx[3 * (size_t)s], cnv[s]);
#pragma omp parallel for schedule(dynamic, 16)
  for (int kk = 0; kk < c->slvmax; ++kk) {
    const int i = c->tagpt[kk];
    if (i == tagslt) continue;
    double* o = out + (size_t)kk * P;
    const double qk = c->mol_charge[i - 1];
    for (int s = 0; s < ns; ++s) {
      const int ats = b + s;  // 1-based atom of solute site s
      const int ts = c->ljtype[ats - 1];
      const double eps_s = c->ljene[(ts - 1) + (size_t)T * (ts - 1)];
      const double sig_s = std::sqrt(c->ljlensq[(ts - 1) + (size_t)T * (ts - 1)]);
      double dq = recpcal_energy(c, tagslt, i, cnv[s]) - resid * qk;
      double deps = 0.0, dsig = 0.0;
      for (int at = c->mbi[i - 1]; at < c->mbi[i]; ++at) {
        double d2 = 0.0;
        for (int a = 0; a < 3; ++a) {
          const double hh = 0.5 * L[a];
          const double d = hh - std::fabs(hh - std::fabs(wrap(c->pos(a + 1, at), a) - wrap(sx[3 * s + a], a)));
          d2 += d * d;
        }
        const int tt = c->ljtype[at - 1];
        const double ljeps = c->ljene[(tt - 1) + (size_t)T * (ts - 1)];
        const double x = c->ljlensq[(tt - 1) + (size_t)T * (ts - 1)];
        if (ljeps > 0.0 && d2 <= k.up2) {
          double vdwa, vdwb;
          lj_parts(c->p, k, x, d2, vdwa, vdwb);
          const double lj = 4.0 * ljeps * (vdwa - vdwb);
          if (eps_s > 0.0) deps += lj / (2.0 * eps_s);
          const double dldx = 4.0 * ljeps * (6.0 * vdwa - 3.0 * vdwb) / x;
          const double dxds = (cmbrule == 0) ? std::sqrt(x) : (sig_s > 0.0 ? x / sig_s : 0.0);
          dsig += dldx * dxds;
        }
        if (d2 <= k.ele2) {
          const double r = std::sqrt(d2);
          dq += c->charge[at - 1] * (1.0 - std::erf(c->p.screen * r)) / r;
        }
      }
      o[3 * s + 0] = dq;
      o[3 * s + 1] = deps;
      o[3 * s + 2] = dsig;
    }
  }
  return ORC_OK;
}

// the intermediate-state extension: bins where refs_density <= tiny (1e-30) form the
// zero-density set read from engref (extensions/Intermediate/engproc.F90:275-318)
int orc_intermediate_enable(orc_ctx* c, const double* refs_density) {
  if (!c || !refs_density || c->ermax <= 0 || c->p.slttype != 1) return ORC_E_PARAM;
  c->do_intermediate = true;
  c->zerodns_crd.assign(c->ermax, 1);
  for (int i = 0; i < c->ermax; ++i)
    if (refs_density[i] > 1.0e-30) c->zerodns_crd[i] = 0;
  c->edintm.assign(c->ermax, 0.0);
  c->uvintm.assign(c->numslv, 0.0);
  c->soln_total = c->soln_intm = c->norm_intm = 0.0;
  return ORC_OK;
}

int orc_intermediate_get(const orc_ctx* c, double* edintm, double* uvintm, double* totals) {
  if (!c || !c->do_intermediate) return ORC_E_PARAM;
  if (edintm) std::copy(c->edintm.begin(), c->edintm.end(), edintm);
  if (uvintm) std::copy(c->uvintm.begin(), c->uvintm.end(), uvintm);
  if (totals) {
    totals[0] = c->soln_total;
    totals[1] = c->soln_intm;
    totals[2] = c->norm_intm;
  }
  return ORC_OK;
}

int orc_direct_ewald(const orc_ctx* c, int tagslt, const double* solute_sitepos, int mmax, double* out,
                     double* self_out) {
  // E(u, j) = sum_{m != 0} exp(-pi^2 |m|^2 / beta^2) / (pi V |m|^2) Re[S_u(m) conj(S_j(m))]
  // with S(m) = sum q exp(2 pi i m.r), m = invcl^T n: the continuum limit of the PME energy.
  if (!c || !c->frame_ready) return ORC_E_PARAM;
  const int ns = c->numsite[tagslt - 1];
  const int b = c->mbi[tagslt - 1];
  std::vector<double> pos = c->sitepos;
  if (solute_sitepos) std::memcpy(&pos[3 * (size_t)(b - 1)], solute_sitepos, sizeof(double) * 3 * ns);
  const double beta = c->p.screen;
  std::vector<double> acc(c->slvmax, 0.0);
  double self = 0.0;
  std::vector<cd> su;
  for (int n3 = -mmax; n3 <= mmax; ++n3)
    for (int n2 = -mmax; n2 <= mmax; ++n2)
      for (int n1 = -mmax; n1 <= mmax; ++n1) {
        if (!n1 && !n2 && !n3) continue;
        const double nv[3] = {(double)n1, (double)n2, (double)n3};
        double m[3];
        for (int a = 0; a < 3; ++a) m[a] = c->invcl[0 + 3 * a] * nv[0] + c->invcl[1 + 3 * a] * nv[1] + c->invcl[2 + 3 * a] * nv[2];
        const double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
        const double f = std::exp(-PI * PI * m2 / (beta * beta)) / (PI * c->volume * m2);
        if (f < 1e-300) continue;
        cd s_u(0, 0);
        for (int a = 0; a < ns; ++a) {
          const double* r = &pos[3 * (size_t)(b - 1 + a)];
          const double ph = 2.0 * PI * (m[0] * r[0] + m[1] * r[1] + m[2] * r[2]);
          s_u += c->charge[b - 1 + a] * cd(std::cos(ph), std::sin(ph));
        }
        self += 0.5 * f * std::norm(s_u);
        for (int k = 0; k < c->slvmax; ++k) {
          const int i = c->tagpt[k];
          if (i == tagslt) continue;
          cd s_j(0, 0);
          for (int a = c->mbi[i - 1]; a < c->mbi[i]; ++a) {
            const double* r = &pos[3 * (size_t)(a - 1)];
            const double ph = 2.0 * PI * (m[0] * r[0] + m[1] * r[1] + m[2] * r[2]);
            s_j += c->charge[a - 1] * cd(std::cos(ph), std::sin(ph));
          }
          acc[k] += f * (s_u * std::conj(s_j)).real();
        }
      }
  std::copy(acc.begin(), acc.end(), out);
  if (self_out) *self_out = self;
  return ORC_OK;
}

}  // extern "C"
