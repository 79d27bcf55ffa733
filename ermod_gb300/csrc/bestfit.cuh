// bestfit.cuh -- best-fit superposition in FP64 (bestfit.F90): mass-weighted centres,
// the rotation that best fits one point set onto another as a unit quaternion (Horn's
// closed form, J. Opt. Soc. Am. A 4, 629 (1987): the eigenvector of the largest
// eigenvalue of a symmetric 4 x 4 matrix of sums of products), rotation by q v q*, and
// RMSDs with and without the fit.
//
// The reference takes the eigenvector from LAPACK dsyev.  Here a cyclic Jacobi iteration
// (the classical method: rotations that zero each off-diagonal element in turn, Golub &
// Van Loan, Matrix Computations, 4th ed., section 8.5) finds it; a unit eigenvector is
// fixed up to its sign, and q and -q give the same rotation, so the fitted coordinates
// agree with the reference's to rounding.
#pragma once

#include <cmath>

namespace ermod {
namespace bestfit {

#ifdef __CUDACC__
#define ERMOD_HD __host__ __device__ __forceinline__
#else
#define ERMOD_HD inline
#endif

// Eigen-decomposition of the symmetric a (overwritten; its diagonal ends as the
// eigenvalues); v receives the eigenvectors as columns.
ERMOD_HD void jacobi4(double a[4][4], double v[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) v[i][j] = (i == j) ? 1.0 : 0.0;
  double norm = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) norm += a[i][j] * a[i][j];
  for (int sweep = 0; sweep < 32; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) off += a[p][q] * a[p][q];
    if (!(off > 1e-32 * norm)) break;  // converged (also stops on NaN input)
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) {
        const double apq = a[p][q];
        if (apq == 0.0) continue;
        // the rotation angle that zeroes a[p][q]: tan of it from cot(2 phi) = theta
        const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
        double t;
        if (std::fabs(theta) > 1e150)
          t = 0.5 / theta;
        else
          t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        // a <- J^T a J, with J the rotation in the (p, q) plane
        for (int k = 0; k < 4; ++k) {
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        a[p][q] = a[q][p] = 0.0;
        for (int k = 0; k < 4; ++k) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
}

// find_rotation_quaternion (bestfit.F90:107-156): S(j, i) = sum_n w_n ref_i(n) moved_j(n)
// of centred points; q = the eigenvector of the largest eigenvalue of Horn's matrix
ERMOD_HD void rotation_quaternion(const double S[3][3], double q[4]) {
  double a[4][4], v[4][4];
  a[0][0] = S[0][0] + S[1][1] + S[2][2];
  a[1][1] = S[0][0] - S[1][1] - S[2][2];
  a[2][2] = -S[0][0] + S[1][1] - S[2][2];
  a[3][3] = -S[0][0] - S[1][1] + S[2][2];
  a[0][1] = a[1][0] = S[1][2] - S[2][1];
  a[0][2] = a[2][0] = S[2][0] - S[0][2];
  a[0][3] = a[3][0] = S[0][1] - S[1][0];
  a[1][2] = a[2][1] = S[0][1] + S[1][0];
  a[2][3] = a[3][2] = S[1][2] + S[2][1];
  a[1][3] = a[3][1] = S[2][0] + S[0][2];
  jacobi4(a, v);
  int best = 0;
  for (int k = 1; k < 4; ++k)
    if (a[k][k] > a[best][best]) best = k;
  for (int i = 0; i < 4; ++i) q[i] = v[i][best];
}

// rotate (bestfit.F90:75-87): q x q* for the unit quaternion q = (q0, q1, q2, q3)
ERMOD_HD void rotate(const double q[4], const double x[3], double out[3]) {
  // t = q (0, x)
  const double t0 = -(q[1] * x[0] + q[2] * x[1] + q[3] * x[2]);
  const double t1 = q[2] * x[2] - q[3] * x[1] + q[0] * x[0];
  const double t2 = q[3] * x[0] - q[1] * x[2] + q[0] * x[1];
  const double t3 = q[1] * x[1] - q[2] * x[0] + q[0] * x[2];
  // out = vector part of t q*, q* = (q0, -q1, -q2, -q3)
  out[0] = (t2 * -q[3] - t3 * -q[2]) + t0 * -q[1] + q[0] * t1;
  out[1] = (t3 * -q[1] - t1 * -q[3]) + t0 * -q[2] + q[0] * t2;
  out[2] = (t1 * -q[2] - t2 * -q[1]) + t0 * -q[3] + q[0] * t3;
}

// The fit of the point set a (weights w) onto ref (fit_a_rotate_b, bestfit.F90:215-242):
// centres cref, ca and the quaternion q; a point b then maps to rotate(q, b - ca) + cref.
// Returns false when the weights sum to zero ('bst_zrw').  Points are read through
// accessors so that callers can pass strided or gathered sets.
template <class RefAt, class AAt, class WAt>
ERMOD_HD bool fit_transform(int n, RefAt ref, AAt a, WAt w, double cref[3], double ca[3], double q[4]) {
  double W = 0.0;
  for (int i = 0; i < 3; ++i) cref[i] = ca[i] = 0.0;
  for (int k = 0; k < n; ++k) W += w(k);
  if (W == 0.0) return false;
  for (int i = 0; i < 3; ++i) {
    double sr = 0.0, sa = 0.0;
    for (int k = 0; k < n; ++k) {
      sr += ref(k, i) * w(k);
      sa += a(k, i) * w(k);
    }
    cref[i] = sr / W;
    ca[i] = sa / W;
  }
  double S[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += (ref(k, i) - cref[i]) * (a(k, j) - ca[j]) * w(k);
      S[j][i] = s;
    }
  rotation_quaternion(S, q);
  return true;
}

ERMOD_HD void apply_fit(const double cref[3], const double ca[3], const double q[4], const double b[3],
                        double out[3]) {
  const double d[3] = {b[0] - ca[0], b[1] - ca[1], b[2] - ca[2]};
  rotate(q, d, out);
  for (int i = 0; i < 3; ++i) out[i] += cref[i];
}

#undef ERMOD_HD

}  // namespace bestfit
}  // namespace ermod
