// host_setup.cpp -- the reference's own host-side set-up arithmetic, exported through the
// C ABI so a host without ERmod's Fortran (the Python front end, a C++ harness) builds
// the same inputs the Fortran host would:
//   ermod_enginit_species   energy-coordinate construction (engproc.F90:163-218)
//   ermod_getscrn           Ewald screening from ewtoler (setconf.F90:515-535)
//   ermod_lj_tables         LJ type deduplication + combination rules (setconf.F90:720-823)
//   ermod_engstore_merge    engstore's rank merge and normalisation (engproc.F90:475-560)
//   ermod_write_*           engstore's output files (engproc.F90:594-657), readable by slvfe
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ermod_gpu.h"

namespace ermod {
void set_error_string(const std::string& s);
}

namespace {
double ipow(double x, int e) {  // x**e for a constant integer exponent, binary powering
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
// Fortran Gw.d output (no exponent width) with gfortran's conventions: values whose
// magnitude, rounded to d significant digits, lies in [0.1, 10^d) are written as
// F(w-4).(d-s) followed by 4 blanks (s = digits before the point); zero as
// F(w-4).(d-1) + 4 blanks; anything else as Ew.d, 0.ddd..E+xx (3-digit exponents
// drop the E).  The digits come from the C library's correctly rounded conversion.
std::string fortran_g(double x, int w, int d) {
  char buf[128];
  if (x == 0.0) {
    std::snprintf(buf, sizeof buf, "%*.*f    ", w - 4, d - 1, x);
    return buf;
  }
  std::snprintf(buf, sizeof buf, "%.*e", d - 1, std::fabs(x));
  const char* ep = std::strchr(buf, 'e');
  const int e10 = std::atoi(ep + 1);
  if (e10 >= -1 && e10 <= d - 1) {
    const int s = e10 + 1;
    std::snprintf(buf, sizeof buf, "%*.*f    ", w - 4, d - s, x);
    return buf;
  }
  std::string digits;
  for (const char* c = buf; c < ep; ++c)
    if (*c >= '0' && *c <= '9') digits += *c;
  const int ex = e10 + 1;  // 0.d1d2... x 10^ex
  char tail[16];
  if (std::abs(ex) <= 99)
    std::snprintf(tail, sizeof tail, "E%c%02d", ex < 0 ? '-' : '+', std::abs(ex));
  else
    std::snprintf(tail, sizeof tail, "%c%03d", ex < 0 ? '-' : '+', std::abs(ex));
  std::string body = std::string(x < 0 ? "-" : "") + "0." + digits + tail;
  if ((int)body.size() > w) body.erase(x < 0 ? 1 : 0, 1);  // drop the optional leading zero
  if ((int)body.size() < w) body.insert(0, (size_t)(w - body.size()), ' ');
  return body;
}

// repval('intn') (engproc.F90:1185-1223): the representative energy of bin iduv (0-based)
double repval_intn(int iduv, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd, int* spec) {
  int idmin = 0, cnt = 0;
  for (cnt = 0; cnt < numslv; ++cnt) {
    if (iduv < idmin + uvmax[cnt]) break;
    idmin += uvmax[cnt];
  }
  if (cnt == numslv) cnt = numslv - 1;
  *spec = cnt + 1;
  const int idpt = iduv - idmin + 1;  // 1-based within the species
  if (idpt <= uvsoft[cnt]) return (uvcrd[iduv] + uvcrd[iduv + 1]) / 2.0;
  if (idpt < uvmax[cnt]) return std::sqrt(uvcrd[iduv] * uvcrd[iduv + 1]);
  return uvcrd[iduv];
}

}  // namespace

extern "C" {

int ermod_format_g(double x, int w, int d, char* out, int cap) {
  if (!out || w <= 4 || d <= 0 || cap <= w) return ERMOD_E_PARAM;
  const std::string s = fortran_g(x, w, d);
  std::snprintf(out, (size_t)cap, "%s", s.c_str());
  return ERMOD_OK;
}

int ermod_write_engdist(const char* path, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd,
                        const double* edens) {
  if (!path || numslv <= 0 || !uvmax || !uvsoft || !uvcrd || !edens) return ERMOD_E_PARAM;
  int ermax = 0;
  for (int i = 0; i < numslv; ++i) ermax += uvmax[i];
  std::FILE* f = std::fopen(path, "w");
  if (!f) {
    ermod::set_error_string(std::string("cannot open ") + path);
    return ERMOD_E_PARAM;
  }
  for (int iduv = 0; iduv < ermax; ++iduv) {  // '(g15.7,i5,g25.15)'
    int pti = 0;
    const double factor = repval_intn(iduv, numslv, uvmax, uvsoft, uvcrd, &pti);
    std::fprintf(f, "%s%5d%s\n", fortran_g(factor, 15, 7).c_str(), pti, fortran_g(edens[iduv], 25, 15).c_str());
  }
  return std::fclose(f) == 0 ? ERMOD_OK : ERMOD_E_PARAM;
}

int ermod_write_selfdist(const char* path, int esmax, const double* escrd, const double* eself) {
  if (!path || esmax <= 0 || !escrd || !eself) return ERMOD_E_PARAM;
  std::FILE* f = std::fopen(path, "w");
  if (!f) {
    ermod::set_error_string(std::string("cannot open ") + path);
    return ERMOD_E_PARAM;
  }
  for (int iduv = 0; iduv < esmax; ++iduv) {  // repval('self'), '(g15.7,g25.15)'
    const double factor = (iduv + 1 < esmax) ? (escrd[iduv] + escrd[iduv + 1]) / 2.0 : escrd[esmax - 1];
    std::fprintf(f, "%s%s\n", fortran_g(factor, 15, 7).c_str(), fortran_g(eself[iduv], 25, 15).c_str());
  }
  return std::fclose(f) == 0 ? ERMOD_OK : ERMOD_E_PARAM;
}

int ermod_write_corr(const char* path, int ermax, const double* ecorr) {
  if (!path || ermax <= 0 || !ecorr) return ERMOD_E_PARAM;
  const uint64_t bytes = (uint64_t)ermax * (uint64_t)ermax * sizeof(double);
  if (bytes > 2147483639ull) {  // one record, one 4-byte marker each side
    ermod::set_error_string("ecorr larger than one 2 GiB unformatted record");
    return ERMOD_E_UNSUPPORTED;
  }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) {
    ermod::set_error_string(std::string("cannot open ") + path);
    return ERMOD_E_PARAM;
  }
  const uint32_t mk = (uint32_t)bytes;
  unsigned char m[4] = {(unsigned char)(mk & 0xff), (unsigned char)((mk >> 8) & 0xff),
                        (unsigned char)((mk >> 16) & 0xff), (unsigned char)(mk >> 24)};  // little endian
  bool ok = std::fwrite(m, 1, 4, f) == 4;
  for (size_t i = 0; ok && i < (size_t)ermax * ermax; ++i) {
    uint64_t v;
    std::memcpy(&v, &ecorr[i], 8);
    unsigned char b[8];
    for (int k = 0; k < 8; ++k) b[k] = (unsigned char)((v >> (8 * k)) & 0xff);
    ok = std::fwrite(b, 1, 8, f) == 8;
  }
  ok = ok && std::fwrite(m, 1, 4, f) == 4;
  return (std::fclose(f) == 0 && ok) ? ERMOD_OK : ERMOD_E_PARAM;
}

int ermod_write_uvrange(const char* path, int numslv, const double* minuv, const double* maxuv) {
  if (!path || numslv <= 0 || !minuv || !maxuv) return ERMOD_E_PARAM;
  std::FILE* f = std::fopen(path, "w");
  if (!f) {
    ermod::set_error_string(std::string("cannot open ") + path);
    return ERMOD_E_PARAM;
  }
  std::fprintf(f, " species     minimum        maximum\n");
  for (int pti = 0; pti <= numslv; ++pti) {
    if (maxuv[pti] < 1.0e5)  // '(i5,2f15.5)'
      std::fprintf(f, "%5d%15.5f%15.5f\n", pti, minuv[pti], maxuv[pti]);
    else  // '(i5,f15.5,g18.5)'
      std::fprintf(f, "%5d%15.5f%s\n", pti, minuv[pti], fortran_g(maxuv[pti], 18, 5).c_str());
  }
  return std::fclose(f) == 0 ? ERMOD_OK : ERMOD_E_PARAM;
}


int ermod_enginit_species(const double* hist, int pecore, int large, double* ercrd_out, int* pemax_out,
                          int* pesoft_out) {
  if (!hist || !ercrd_out || !pemax_out || !pesoft_out || large <= 0 || pecore < 0) return ERMOD_E_PARAM;
  double ecdmin = hist[0], ecfmns = hist[1];
  const double ecdcen = hist[2];
  double eccore = hist[3];
  const double ecdmax = hist[4], eclbin = hist[5], ecfbin = hist[6], ec0bin = hist[7], finfac = hist[8];
  const int rglmax = 5;
  // the "margin" shift of the low-energy side and the symmetric fine region
  const double ectmvl = finfac * ecfbin;
  ecdmin = ecdmin - ectmvl;
  ecfmns = ecfmns - ectmvl;
  const double ecmns0 = ecdcen - ectmvl;
  const double ecpls0 = 2.0 * ecdcen - ecmns0;
  const double ecfpls = 2.0 * ecdcen - ecfmns;
  eccore = eccore + ecfpls - ecdcen;
  const double region_edge[rglmax + 2] = {ecdmin, ecfmns, ecmns0, ecpls0, ecfpls, eccore, ecdmax};
  int first_index[rglmax + 2];
  first_index[0] = 1;
  for (int regn = 1; regn <= rglmax; ++regn) {
    const double step = (regn == 1 || regn == 5) ? eclbin : ((regn == 2 || regn == 4) ? ecfbin : ec0bin);
    const double width = region_edge[regn] - region_edge[regn - 1];
    if (width < step) {
      ermod::set_error_string("eng_ecd: an energy-coordinate region is narrower than its bin width");
      return ERMOD_E_PARAM;
    }
    first_index[regn] = first_index[regn - 1] + (int)std::lround(width / step);
  }
  const int pesoft = first_index[rglmax] - first_index[0];
  const int pemax = pesoft + pecore;
  first_index[rglmax + 1] = pemax;
  if (pemax > large) {
    ermod::set_error_string("eng_siz: the number of energy-coordinate meshes is too large");
    return ERMOD_E_PARAM;
  }
  std::vector<double> crd(large + 2, 0.0);  // 1-based like ercrd(:, pti)
  for (int r = 0; r <= rglmax + 1; ++r) crd[first_index[r]] = region_edge[r];
  const int nregion = (pecore == 0) ? rglmax : rglmax + 1;
  for (int regn = 1; regn <= nregion; ++regn) {
    const int lo = first_index[regn - 1], hi = first_index[regn];
    const bool logarithmic = (regn == rglmax + 1);
    const double span = logarithmic ? std::log(crd[hi] / crd[lo]) : crd[hi] - crd[lo];
    const double per_bin = span / (double)(hi - lo);
    for (int i = lo; i <= hi - 1; ++i) {
      const double off = per_bin * (double)(i - lo);
      crd[i] = logarithmic ? crd[lo] * std::exp(off) : crd[lo] + off;
    }
  }
  for (int i = 1; i <= pemax; ++i) ercrd_out[i - 1] = crd[i];
  *pemax_out = pemax;
  *pesoft_out = pesoft;
  return ERMOD_OK;
}

double ermod_getscrn(double ewtoler, double elecut, int distance_form) {
  // bisection on erfc(alpha rc) [/ rc] = ewtoler, as the reference iterates it
  const double tol = 1.0e-20;
  double gap = tol + 1.0, lo = 0.0, hi = 1.0e3, alpha = 0.0;
  while (gap > tol) {
    alpha = (lo + hi) / 2.0;
    double f = std::erfc(alpha * elecut);
    if (distance_form) f = f / elecut;
    if (f > ewtoler)
      lo = alpha;
    else
      hi = alpha;
    gap = std::fabs(f - ewtoler);
  }
  return alpha;
}

int ermod_lj_tables(int nsite, const double* eps_in, const double* len_in, int ljformat, int cmbrule, int max_types,
                    int* ljtype, int* ljtype_max, double* ljene_mat, double* ljlensq_mat) {
  if (nsite <= 0 || !eps_in || !len_in || !ljtype || !ljtype_max || !ljene_mat || !ljlensq_mat || max_types <= 0)
    return ERMOD_E_PARAM;
  if (ljformat < 0 || ljformat > 4 || cmbrule < 0 || cmbrule > 1) return ERMOD_E_PARAM;
  const double rmin_half_to_sigma = 1.7817974362806784;  // 2^(5/6)
  const double nm_to_angstrom = 10.0, kj_to_kcal = 1.0 / 4.184;
  std::vector<double> tab_len, tab_eps;
  for (int s = 0; s < nsite; ++s) {
    double e = eps_in[s], l = len_in[s];
    if (ljformat == 1) l = rmin_half_to_sigma * l;
    if (ljformat == 3 || ljformat == 4) {  // (A, C) -> (eps, sigma)
      if (l != 0.0) {
        const double sigma = std::pow(e / l, 1.0 / 6.0);
        e = l / (4.0 * ipow(sigma, 6));
        l = sigma;
      } else {
        e = 0.0;
      }
    }
    if (ljformat == 2 || ljformat == 4) {
      e = kj_to_kcal * e;
      l = nm_to_angstrom * l;
    }
    int found = 0;
    for (size_t t = 0; t < tab_len.size(); ++t)
      if (tab_len[t] == l && tab_eps[t] == e) {
        found = (int)t + 1;
        break;
      }
    if (!found) {
      if ((int)tab_len.size() >= max_types) return ERMOD_E_PARAM;
      tab_len.push_back(l);
      tab_eps.push_back(e);
      found = (int)tab_len.size();
    }
    ljtype[s] = found;
  }
  const int n = (int)tab_len.size();
  *ljtype_max = n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double ls = (cmbrule == 0) ? ((tab_len[j] + tab_len[i]) / 2.0) * ((tab_len[j] + tab_len[i]) / 2.0)
                                       : tab_len[j] * tab_len[i];
      ljlensq_mat[j + (size_t)n * i] = ls;
      ljene_mat[j + (size_t)n * i] = std::sqrt(tab_eps[j] * tab_eps[i]);
    }
  return ERMOD_OK;
}

int ermod_engstore_merge(int nrank, int slttype, int wgtslf, double temp, int ermax, int esmax, int numslv,
                         double* edens, double* ecorr, double* eself, double* slnuv, double* minuv, double* maxuv,
                         double* scalars) {
  if (nrank <= 0 || !edens || !scalars || !minuv || !maxuv) return ERMOD_E_PARAM;
  const size_t E = (size_t)ermax, E2 = E * E;
  if (wgtslf && nrank > 1) {
    double vmax = -1.0e300;
    for (int r = 0; r < nrank; ++r) vmax = std::fmax(vmax, scalars[5 * r + 3]);
    for (int r = 0; r < nrank; ++r) {
      double vl = scalars[5 * r + 3];
      if (scalars[5 * r + 4] == 0.0) vl = vmax;  // uninitialised ranks take the global offset
      const double sc = (slttype == 1) ? std::exp((vl - vmax) / temp) : std::exp(-(vl - vmax) / temp);
      scalars[5 * r + 0] *= sc;
      if (eself)
        for (int i = 0; i < esmax; ++i) eself[(size_t)r * esmax + i] *= sc;
      if (slnuv && slttype == 1)
        for (int i = 0; i < numslv; ++i) slnuv[(size_t)r * numslv + i] *= sc;
      for (size_t i = 0; i < E; ++i) edens[r * E + i] *= sc;
      if (ecorr)
        for (size_t i = 0; i < E2; ++i) ecorr[r * E2 + i] *= sc;
    }
    scalars[3] = vmax;
  }
  for (int r = 1; r < nrank; ++r) {
    for (int k = 0; k < 3; ++k) scalars[k] += scalars[5 * r + k];
    if (eself)
      for (int i = 0; i < esmax; ++i) eself[i] += eself[(size_t)r * esmax + i];
    if (slnuv && slttype == 1)
      for (int i = 0; i < numslv; ++i) slnuv[i] += slnuv[(size_t)r * numslv + i];
    for (int i = 0; i <= numslv; ++i) {
      minuv[i] = std::fmin(minuv[i], minuv[(size_t)r * (numslv + 1) + i]);
      maxuv[i] = std::fmax(maxuv[i], maxuv[(size_t)r * (numslv + 1) + i]);
    }
    for (size_t i = 0; i < E; ++i) edens[i] += edens[r * E + i];
    if (ecorr)
      for (size_t i = 0; i < E2; ++i) ecorr[i] += ecorr[r * E2 + i];
  }
  const double engnorm = scalars[0];
  for (size_t i = 0; i < E; ++i) edens[i] = edens[i] / engnorm;
  if (ecorr)
    for (size_t i = 0; i < E2; ++i) ecorr[i] = ecorr[i] / engnorm;
  if (eself)
    for (int i = 0; i < esmax; ++i) eself[i] = eself[i] / engnorm;
  scalars[2] = scalars[2] / engnorm;
  return ERMOD_OK;
}

}  // extern "C"
