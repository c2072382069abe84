/*
 * dqmc_oracle.cpp — CPU oracle for the DQMC sweep hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see dqmc_oracle.h).  A restatement, written from
 * the reference's algorithm, of:
 *   src/dqmc_walker.cpp:109-412            walker set-up and half-sweeps
 *   src/model/repulsive_hubbard.cpp:44-243  ratio, rank-1 update, B products
 *   src/model/attractive_hubbard.cpp:44-245 (attractive variant)
 *   src/model/model_base.cpp:7-35           dense exp(-dtau K) products
 *   src/checkerboard/square.cpp:28-226      checkerboard break-up
 *   src/svd_stack.cpp:34-87                 UDV stack
 *   include/utils/numerical_stable.hpp:34-239  stable (1 + L R^T)^-1
 *   include/utils/linear_algebra.hpp:41-80  dgesvd semantics (U, S desc, V)
 *   src/lattice/square.cpp:31-178           square lattice tables (hopping matrix zeroed)
 *   src/lattice/cubic.cpp:35-219            cubic lattice tables (dense K only)
 *   src/measure/measure_methods.cpp:22-255  equal-time observables
 *   src/measure/measure_handler.cpp:170-240 bin normalisation
 * Third-party arithmetic replaced here: Eigen 3.4 GEMM / PartialPivLU /
 * FullPivHouseholderQR / MatrixFunctions::exp and MKL LAPACKE_dgesvd.  The
 * oracle uses its own FP64 routines (or scipy's LAPACK when hooked).
 */
#include "dqmc_oracle.h"

#include <algorithm>
#include <array>
#include <cassert>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <vector>

namespace {

using Vec = std::vector<double>;

orc_dgemm_t g_dgemm = nullptr;
orc_dgesvd_t g_dgesvd = nullptr;

// ----------------------------------------------------------------------------
// Dense column-major helpers (n x n)
// ----------------------------------------------------------------------------
inline double& at(Vec& a, int n, int r, int c) { return a[(size_t)r + (size_t)c * n]; }
inline double at(const Vec& a, int n, int r, int c) { return a[(size_t)r + (size_t)c * n]; }

Vec identity(int n) {
  Vec a((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) at(a, n, i, i) = 1.0;
  return a;
}

Vec transpose(const Vec& a, int n) {
  Vec t((size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) at(t, n, c, r) = at(a, n, r, c);
  return t;
}

// C = op(A) op(B), square n.
Vec gemm(char ta, char tb, int n, const Vec& A, const Vec& B) {
  Vec C((size_t)n * n, 0.0);
  if (g_dgemm) {
    const double one = 1.0, zero = 0.0;
    g_dgemm(&ta, &tb, &n, &n, &n, &one, A.data(), &n, B.data(), &n, &zero, C.data(), &n);
    return C;
  }
  const Vec Ab = (ta == 'T') ? transpose(A, n) : A;
  const Vec Bb = (tb == 'T') ? transpose(B, n) : B;
  for (int j = 0; j < n; ++j) {
    double* cj = &C[(size_t)j * n];
    for (int k = 0; k < n; ++k) {
      const double b = Bb[(size_t)k + (size_t)j * n];
      const double* ak = &Ab[(size_t)k * n];
      for (int i = 0; i < n; ++i) cj[i] += ak[i] * b;
    }
  }
  return C;
}

// ----------------------------------------------------------------------------
// Symmetric eigen-decomposition (cyclic Jacobi) for exp(-dtau K).
// Replaces Eigen's MatrixFunctions::exp used at repulsive_hubbard.cpp:64-65;
// K is symmetric so exp(x K) = V diag(exp(x lambda)) V^T is exact in theory.
// ----------------------------------------------------------------------------
void sym_eig(int n, Vec a, Vec& w, Vec& v) {
  v = identity(n);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int c = 0; c < n; ++c)
      for (int r = 0; r < n; ++r) {
        if (r != c) off += at(a, n, r, c) * at(a, n, r, c);
        else diag += at(a, n, r, c) * at(a, n, r, c);
      }
    if (off <= 1e-32 * (diag + off) || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = at(a, n, p, q);
        if (apq == 0.0) continue;
        const double app = at(a, n, p, p), aqq = at(a, n, q, q);
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // columns p,q
          const double akp = at(a, n, k, p), akq = at(a, n, k, q);
          at(a, n, k, p) = c * akp - s * akq;
          at(a, n, k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p,q
          const double apk = at(a, n, p, k), aqk = at(a, n, q, k);
          at(a, n, p, k) = c * apk - s * aqk;
          at(a, n, q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = at(v, n, k, p), vkq = at(v, n, k, q);
          at(v, n, k, p) = c * vkp - s * vkq;
          at(v, n, k, q) = s * vkp + c * vkq;
        }
      }
  }
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) w[i] = at(a, n, i, i);
}

Vec sym_exp(int n, const Vec& k, double x) {
  Vec w, v;
  sym_eig(n, k, w, v);
  Vec out((size_t)n * n, 0.0);
  for (int m = 0; m < n; ++m) {
    const double e = std::exp(x * w[m]);
    for (int c = 0; c < n; ++c) {
      const double vc = at(v, n, c, m) * e;
      for (int r = 0; r < n; ++r) at(out, n, r, c) += at(v, n, r, m) * vc;
    }
  }
  return out;
}

// ----------------------------------------------------------------------------
// SVD  A = U diag(S) V^T, S descending (LAPACKE_dgesvd('A','A') semantics of
// include/utils/linear_algebra.hpp:41-80).  Own routine: one-sided Jacobi
// (Hestenes 1958; Demmel & Veselic 1992), accurate for column-graded input.
// ----------------------------------------------------------------------------
void svd_jacobi(int n, const Vec& A, Vec& U, Vec& S, Vec& V) {
  Vec W = A;
  V = identity(n);
  const double eps = 2.220446049250313e-16;
  for (int sweep = 0; sweep < 80; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double a = 0, b = 0, g = 0;
        const double* wp = &W[(size_t)p * n];
        const double* wq = &W[(size_t)q * n];
        for (int k = 0; k < n; ++k) { a += wp[k] * wp[k]; b += wq[k] * wq[k]; g += wp[k] * wq[k]; }
        if (g == 0.0 || std::fabs(g) <= eps * std::sqrt(a) * std::sqrt(b)) continue;
        rotated = true;
        const double zeta = (b - a) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        double* wpm = &W[(size_t)p * n];
        double* wqm = &W[(size_t)q * n];
        for (int k = 0; k < n; ++k) {
          const double x = wpm[k], y = wqm[k];
          wpm[k] = c * x - s * y;
          wqm[k] = s * x + c * y;
        }
        double* vp = &V[(size_t)p * n];
        double* vq = &V[(size_t)q * n];
        for (int k = 0; k < n; ++k) {
          const double x = vp[k], y = vq[k];
          vp[k] = c * x - s * y;
          vq[k] = s * x + c * y;
        }
      }
    if (!rotated) break;
  }
  std::vector<int> idx(n);
  Vec nrm(n);
  for (int j = 0; j < n; ++j) {
    double s = 0;
    for (int k = 0; k < n; ++k) s += at(W, n, k, j) * at(W, n, k, j);
    nrm[j] = std::sqrt(s);
    idx[j] = j;
  }
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return nrm[x] > nrm[y]; });
  U.assign((size_t)n * n, 0.0);
  S.assign(n, 0.0);
  Vec V2((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    const int o = idx[j];
    S[j] = nrm[o];
    for (int k = 0; k < n; ++k) {
      at(U, n, k, j) = nrm[o] > 0 ? at(W, n, k, o) / nrm[o] : (k == j ? 1.0 : 0.0);
      at(V2, n, k, j) = at(V, n, k, o);
    }
  }
  V = V2;
}

void svd(int n, const Vec& A, Vec& U, Vec& S, Vec& V) {
  if (g_dgesvd) {
    Vec a = A, vt((size_t)n * n);
    U.assign((size_t)n * n, 0.0);
    S.assign(n, 0.0);
    int info = 0, lwork = -1;
    double wq = 0;
    const char job = 'A';
    g_dgesvd(&job, &job, &n, &n, a.data(), &n, S.data(), U.data(), &n, vt.data(), &n, &wq, &lwork, &info);
    lwork = (int)wq;
    Vec work(std::max(1, lwork));
    g_dgesvd(&job, &job, &n, &n, a.data(), &n, S.data(), U.data(), &n, vt.data(), &n, work.data(), &lwork,
             &info);
    if (info != 0) throw std::runtime_error("dgesvd failed to converge");
    V = transpose(vt, n);
    return;
  }
  svd_jacobi(n, A, U, S, V);
}

// ----------------------------------------------------------------------------
// Householder QR with column pivoting:  A P = Q R.  Returned as the UDT
// triple U = Q, D = |diag R|, T = D^-1 R P^T so that A = U diag(D) T.
// This is the device algorithm's factorisation (Businger & Golub 1965).
// ----------------------------------------------------------------------------
void qrp_udt(int n, const Vec& A, Vec& U, Vec& D, Vec& T) {
  Vec R = A;
  std::vector<int> piv(n);
  for (int j = 0; j < n; ++j) piv[j] = j;
  Vec tau(n, 0.0);
  for (int k = 0; k < n; ++k) {
    // pivot: largest remaining column norm (recomputed exactly)
    int best = k;
    double bestn = -1.0;
    for (int j = k; j < n; ++j) {
      double s = 0;
      for (int r = k; r < n; ++r) s += at(R, n, r, j) * at(R, n, r, j);
      if (s > bestn) { bestn = s; best = j; }
    }
    if (best != k) {
      for (int r = 0; r < n; ++r) std::swap(at(R, n, r, k), at(R, n, r, best));
      std::swap(piv[k], piv[best]);
    }
    // Householder reflector for R[k:,k]
    double xnorm2 = 0;
    for (int r = k + 1; r < n; ++r) xnorm2 += at(R, n, r, k) * at(R, n, r, k);
    const double alpha = at(R, n, k, k);
    if (xnorm2 == 0.0) { tau[k] = 0.0; continue; }
    const double norm = std::sqrt(alpha * alpha + xnorm2);
    const double beta = alpha >= 0 ? -norm : norm;
    tau[k] = (beta - alpha) / beta;
    const double scal = 1.0 / (alpha - beta);
    for (int r = k + 1; r < n; ++r) at(R, n, r, k) *= scal;
    at(R, n, k, k) = beta;
    // apply H = I - tau v v^T (v[k] = 1) to the trailing columns
    for (int j = k + 1; j < n; ++j) {
      double w = at(R, n, k, j);
      for (int r = k + 1; r < n; ++r) w += at(R, n, r, k) * at(R, n, r, j);
      w *= tau[k];
      at(R, n, k, j) -= w;
      for (int r = k + 1; r < n; ++r) at(R, n, r, j) -= w * at(R, n, r, k);
    }
  }
  // Q = H_0 H_1 ... H_{n-1} applied to I (backward accumulation)
  U = identity(n);
  for (int k = n - 1; k >= 0; --k) {
    if (tau[k] == 0.0) continue;
    for (int j = k; j < n; ++j) {
      double w = at(U, n, k, j);
      for (int r = k + 1; r < n; ++r) w += at(R, n, r, k) * at(U, n, r, j);
      w *= tau[k];
      at(U, n, k, j) -= w;
      for (int r = k + 1; r < n; ++r) at(U, n, r, j) -= w * at(R, n, r, k);
    }
  }
  D.assign(n, 0.0);
  T.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) D[i] = std::fabs(at(R, n, i, i));
  for (int k = 0; k < n; ++k)       // column k of R goes to column piv[k] of T
    for (int i = 0; i <= k; ++i) at(T, n, i, piv[k]) = at(R, n, i, k) / D[i];
}

// ----------------------------------------------------------------------------
// LU with partial pivoting (Eigen PartialPivLU semantics), in place.
// ----------------------------------------------------------------------------
void lu_factor(int n, Vec& a, std::vector<int>& piv, int& nswaps) {
  piv.assign(n, 0);
  nswaps = 0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double m = std::fabs(at(a, n, k, k));
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(at(a, n, r, k)) > m) { m = std::fabs(at(a, n, r, k)); p = r; }
    piv[k] = p;
    if (p != k) {
      ++nswaps;
      for (int c = 0; c < n; ++c) std::swap(at(a, n, k, c), at(a, n, p, c));
    }
    const double d = at(a, n, k, k);
    if (d == 0.0) continue;
    for (int r = k + 1; r < n; ++r) at(a, n, r, k) /= d;
    for (int c = k + 1; c < n; ++c) {
      const double akc = at(a, n, k, c);
      if (akc == 0.0) continue;
      for (int r = k + 1; r < n; ++r) at(a, n, r, c) -= at(a, n, r, k) * akc;
    }
  }
}

// Solve (LU) X = B in place for n_rhs columns.
void lu_solve(int n, const Vec& lu, const std::vector<int>& piv, Vec& b, int nrhs) {
  for (int j = 0; j < nrhs; ++j) {
    double* x = &b[(size_t)j * n];
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int k = 0; k < n; ++k) {
      const double xk = x[k];
      if (xk == 0.0) continue;
      for (int r = k + 1; r < n; ++r) x[r] -= at(lu, n, r, k) * xk;
    }
    for (int k = n - 1; k >= 0; --k) {
      x[k] /= at(lu, n, k, k);
      const double xk = x[k];
      for (int r = 0; r < k; ++r) x[r] -= at(lu, n, r, k) * xk;
    }
  }
}

Vec inverse(int n, const Vec& a) {
  Vec lu = a;
  std::vector<int> piv;
  int ns;
  lu_factor(n, lu, piv, ns);
  Vec x = identity(n);
  lu_solve(n, lu, piv, x, n);
  return x;
}

double det_sign(int n, const Vec& a) {
  Vec lu = a;
  std::vector<int> piv;
  int ns;
  lu_factor(n, lu, piv, ns);
  double s = (ns % 2) ? -1.0 : 1.0;
  for (int i = 0; i < n; ++i) s *= (at(lu, n, i, i) >= 0 ? 1.0 : -1.0);
  return s;
}

// ----------------------------------------------------------------------------
// Full-pivoting Householder QR solve  H X = B  (Eigen fullPivHouseholderQr,
// used at include/utils/numerical_stable.hpp:151).  At step k the largest
// |entry| of the trailing block is moved to (k,k) by a row and a column swap.
// ----------------------------------------------------------------------------
Vec fullpiv_qr_solve(int n, const Vec& H, const Vec& B) {
  Vec a = H, x = B;
  std::vector<int> colp(n);
  for (int j = 0; j < n; ++j) colp[j] = j;
  Vec tau(n, 0.0);
  for (int k = 0; k < n; ++k) {
    int br = k, bc = k;
    double bm = -1;
    for (int c = k; c < n; ++c)
      for (int r = k; r < n; ++r)
        if (std::fabs(at(a, n, r, c)) > bm) { bm = std::fabs(at(a, n, r, c)); br = r; bc = c; }
    if (br != k) {
      for (int c = 0; c < n; ++c) std::swap(at(a, n, k, c), at(a, n, br, c));
      for (int c = 0; c < n; ++c) std::swap(at(x, n, k, c), at(x, n, br, c));
    }
    if (bc != k) {
      for (int r = 0; r < n; ++r) std::swap(at(a, n, r, k), at(a, n, r, bc));
      std::swap(colp[k], colp[bc]);
    }
    double xnorm2 = 0;
    for (int r = k + 1; r < n; ++r) xnorm2 += at(a, n, r, k) * at(a, n, r, k);
    if (xnorm2 == 0.0) continue;
    const double alpha = at(a, n, k, k);
    const double norm = std::sqrt(alpha * alpha + xnorm2);
    const double beta = alpha >= 0 ? -norm : norm;
    tau[k] = (beta - alpha) / beta;
    const double scal = 1.0 / (alpha - beta);
    for (int r = k + 1; r < n; ++r) at(a, n, r, k) *= scal;
    at(a, n, k, k) = beta;
    auto apply = [&](Vec& m, int j) {
      double w = at(m, n, k, j);
      for (int r = k + 1; r < n; ++r) w += at(a, n, r, k) * at(m, n, r, j);
      w *= tau[k];
      at(m, n, k, j) -= w;
      for (int r = k + 1; r < n; ++r) at(m, n, r, j) -= w * at(a, n, r, k);
    };
    for (int j = k + 1; j < n; ++j) apply(a, j);
    for (int j = 0; j < n; ++j) apply(x, j);
  }
  // back substitution R y = Q^T b, then undo the column permutation
  Vec out((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    Vec y(n);
    for (int r = 0; r < n; ++r) y[r] = at(x, n, r, j);
    for (int k = n - 1; k >= 0; --k) {
      y[k] /= at(a, n, k, k);
      for (int r = 0; r < k; ++r) y[r] -= at(a, n, r, k) * y[k];
    }
    for (int k = 0; k < n; ++k) at(out, n, colp[k], j) = y[k];
  }
  return out;
}

// ----------------------------------------------------------------------------
// Stable Green's functions (include/utils/numerical_stable.hpp)
// ----------------------------------------------------------------------------
double matrix_compare_error(int n, const Vec& a, const Vec& b) {  // :34-47
  double e = 0.0;
  for (size_t k = 0; k < (size_t)n * n; ++k) e = std::max(e, std::fabs(a[k] - b[k]));
  return e;
}

void split_max_min(const Vec& d, Vec& dmax, Vec& dmin) {  // :57-71
  const int n = (int)d.size();
  dmax.assign(n, 1.0);
  dmin.assign(n, 1.0);
  for (int i = 0; i < n; ++i) {
    if (d[i] >= 1.0) { dmax[i] = d[i]; dmin[i] = 1.0; }
    else { dmax[i] = 1.0; dmin[i] = d[i]; }
  }
}

// zmat(j,i) = sum_k vmat(j,k) umat(k,i) / dvec(k)   (:79-98)
Vec mult_v_invd_u(int n, const Vec& vmat, const Vec& dvec, const Vec& umat) {
  Vec z((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += at(vmat, n, j, k) * at(umat, n, k, i) / dvec[k];
      at(z, n, j, i) = s;
    }
  return z;
}

// (1 + U S V^T)^-1 via full-pivot QR (:132-152)
Vec greens_00_bb(int n, const Vec& U, const Vec& S, const Vec& V) {
  Vec sbi(n), ss(n);
  for (int i = 0; i < n; ++i) {
    if (S[i] > 1) { sbi[i] = 1.0 / S[i]; ss[i] = 1.0; }
    else { sbi[i] = 1.0; ss[i] = S[i]; }
  }
  Vec H((size_t)n * n), rhs((size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) {
      at(rhs, n, r, c) = sbi[r] * at(U, n, c, r);
      at(H, n, r, c) = sbi[r] * at(U, n, c, r) + ss[r] * at(V, n, c, r);
    }
  return fullpiv_qr_solve(n, H, rhs);
}

// Device-algorithm form: (1 + U D F)^-1 = (Dmax^-1 U^T + Dmin F)^-1 Dmax^-1 U^T, LU solve.
Vec greens_udf(int n, const Vec& U, const Vec& D, const Vec& F) {
  Vec dmax, dmin;
  split_max_min(D, dmax, dmin);
  Vec H((size_t)n * n), rhs((size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) {
      at(rhs, n, r, c) = at(U, n, c, r) / dmax[r];
      at(H, n, r, c) = at(U, n, c, r) / dmax[r] + dmin[r] * at(F, n, r, c);
    }
  std::vector<int> piv;
  int ns;
  lu_factor(n, H, piv, ns);
  lu_solve(n, H, piv, rhs, n);
  return rhs;
}

// ----------------------------------------------------------------------------
// UDV stack (src/svd_stack.cpp:34-87).  Each level keeps U, D and the
// cumulative right factor F (Pi = U diag(D) F).  SVD mode: F = (V0 V1..Vk)^T,
// the product the reference recomputes in MatrixV() (svd_stack.cpp:80-87);
// keeping it cumulative gives the same matrix without the O(k) re-product.
// QRP mode: F = T_k ... T_1 T_0.
// ----------------------------------------------------------------------------
struct Level {
  Vec U, D, F, Vcum;
};

struct Stack {
  int n = 0;
  int kind = ORC_STACK_SVD;
  std::vector<Level> lv;
  int len = 0;
  void init(int n_, int cap, int kind_) {
    n = n_;
    kind = kind_;
    lv.assign(cap, Level{});
    len = 0;
  }
  bool empty() const { return len == 0; }
  void pop() {
    assert(len > 0);
    --len;
  }
  void push(const Vec& m) {  // svd_stack.cpp:34-61
    assert(len < (int)lv.size());
    Vec x;
    if (len == 0) {
      x = m;
    } else {
      const Level& top = lv[len - 1];
      x = gemm('N', 'N', n, m, top.U);  // (matrix * U) * diag(S): order matters
      for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) at(x, n, r, c) *= top.D[c];
    }
    Level& L = lv[len];
    if (kind == ORC_STACK_SVD) {
      Vec V;
      svd(n, x, L.U, L.D, V);
      L.Vcum = (len == 0) ? V : gemm('N', 'N', n, lv[len - 1].Vcum, V);
      L.F = transpose(L.Vcum, n);
    } else {
      Vec T;
      qrp_udt(n, x, L.U, L.D, T);
      L.F = (len == 0) ? T : gemm('N', 'N', n, T, lv[len - 1].F);
    }
    ++len;
  }
  const Level& top() const { return lv[len - 1]; }
};

// compute_equaltime_greens (numerical_stable.hpp:186-239) for both stack kinds.
Vec equaltime_greens(int n, const Stack& left, const Stack& right) {
  if (left.kind == ORC_STACK_SVD) {
    if (left.empty()) {
      const Level& r = right.top();
      return greens_00_bb(n, r.Vcum, r.D, r.U);
    }
    if (right.empty()) {
      const Level& l = left.top();
      return greens_00_bb(n, l.U, l.D, l.Vcum);
    }
  } else {
    if (left.empty()) {  // (1 + F^T D U^T)^-1 = [(1 + U D F)^-1]^T
      const Level& r = right.top();
      return transpose(greens_udf(n, r.U, r.D, r.F), n);
    }
    if (right.empty()) {
      const Level& l = left.top();
      return greens_udf(n, l.U, l.D, l.F);
    }
  }
  const Level& l = left.top();
  const Level& r = right.top();
  Vec dlmax, dlmin, drmax, drmin;
  split_max_min(l.D, dlmax, dlmin);
  split_max_min(r.D, drmax, drmin);
  Vec A = gemm('T', 'N', n, l.U, r.U);
  Vec B = gemm('N', 'T', n, l.F, r.F);  // SVD mode: vl^T vr
  Vec M((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      at(M, n, i, j) = at(A, n, i, j) / (dlmax[i] * drmax[j]) + at(B, n, i, j) * dlmin[i] * drmin[j];
  if (left.kind == ORC_STACK_SVD) {
    const Vec inv = inverse(n, M);
    const Vec a2 = mult_v_invd_u(n, r.U, drmax, inv);
    return mult_v_invd_u(n, a2, dlmax, transpose(l.U, n));
  }
  // device form: G = (U_R Drmax^-1) [M^-1 (Dlmax^-1 U_L^T)]
  Vec rhs((size_t)n * n);
  for (int c = 0; c < n; ++c)
    for (int r2 = 0; r2 < n; ++r2) at(rhs, n, r2, c) = at(l.U, n, c, r2) / dlmax[r2];
  std::vector<int> piv;
  int ns;
  lu_factor(n, M, piv, ns);
  lu_solve(n, M, piv, rhs, n);
  Vec ur = r.U;
  for (int c = 0; c < n; ++c)
    for (int r2 = 0; r2 < n; ++r2) at(ur, n, r2, c) /= drmax[c];
  return gemm('N', 'N', n, ur, rhs);
}

// ----------------------------------------------------------------------------
// Square and cubic lattice tables (src/lattice/square.cpp:31-178,
// src/lattice/cubic.cpp:35-219).  Site i has coordinates x = i % L,
// y = (i / L) % L, z = i / L^2; a displacement is stored as the site index of
// its vector, each component taken mod L.
// ----------------------------------------------------------------------------
struct Lattice {
  int L = 0, dim = 2, N = 0, nk = 0, m_point = 0;  // m_point: the last k star, (pi, ..., pi)
  std::vector<int> nn;  // [i][2 dim]: +x, +y (, +z), then -x, -y (, -z) (square.cpp:69-85, cubic.cpp:84-109)
  Vec hop;              // N x N
  std::vector<double> kx, ky, kz;
  int coord(int i, int a) const { return a == 0 ? i % L : a == 1 ? (i / L) % L : i / (L * L); }
  // displacement from site i to site j (square.cpp:88-105, cubic.cpp:112-132)
  int disp(int i, int j) const {
    int d = 0, w = 1;
    for (int a = 0; a < dim; ++a, w *= L) d += ((coord(j, a) - coord(i, a) + L) % L) * w;
    return d;
  }
  // the site at displacement d from site i (disp(i, shift(i, d)) == d)
  int shift(int i, int d) const {
    int j = 0, w = 1;
    for (int a = 0; a < dim; ++a, w *= L) j += ((coord(i, a) + coord(d, a)) % L) * w;
    return j;
  }
  // Re exp(-i k.r) (square.cpp:148-161, cubic.cpp:186-200)
  double fourier(int d, int k) const {
    if (dim == 2) return std::cos(-coord(d, 0) * kx[k] - coord(d, 1) * ky[k]);
    return std::cos(-coord(d, 0) * kx[k] - coord(d, 1) * ky[k] - coord(d, 2) * kz[k]);
  }
  void init(int L_, int dim_) {
    L = L_;
    dim = dim_;
    N = dim == 2 ? L * L : L * L * L;
    const int nd = 2 * dim;
    nn.assign((size_t)N * nd, 0);
    for (int i = 0; i < N; ++i)
      for (int a = 0, w = 1; a < dim; ++a, w *= L) {
        const int c = coord(i, a);
        nn[i * nd + a] = i + ((c + 1) % L - c) * w;
        nn[i * nd + dim + a] = i + ((c - 1 + L) % L - c) * w;
      }
    hop.assign((size_t)N * N, 0.0);  // zeroed: the reference resizes without init (square.cpp:166)
    for (int i = 0; i < N; ++i)
      for (int a = 0; a < dim; ++a) {
        const int j = nn[i * nd + a];
        at(hop, N, i, j) += 1.0;
        at(hop, N, j, i) += 1.0;
      }
    kx.clear();
    ky.clear();
    kz.clear();
    const auto mom = [&](int i) { return (double)i / L * 2 * M_PI - M_PI; };
    const int lo = (L + 1) / 2;  // ceil(L/2)
    if (dim == 2) {
      for (int i = lo; i <= L; ++i)
        for (int j = lo; j <= i; ++j) {
          kx.push_back(mom(i));
          ky.push_back(mom(j));
        }
    } else {  // the tetrahedron (0,0,0), (pi,0,0), (pi,pi,0), (pi,pi,pi); z outermost (cubic.cpp:47-81)
      for (int k = lo; k <= L; ++k)
        for (int i = k; i <= L; ++i)
          for (int j = k; j <= i; ++j) {
            kx.push_back(mom(i));
            ky.push_back(mom(j));
            kz.push_back(mom(k));
          }
    }
    nk = (int)kx.size();
    m_point = nk - 1;
  }
};

// ----------------------------------------------------------------------------
// Walker + model
// ----------------------------------------------------------------------------
struct Oracle {
  orc_params p{};
  Lattice lat;
  int N = 0, Lt = 0, pace = 0, nstack = 0;
  double dtau = 0, alpha = 0;
  Vec expK, invK, transK;         // dense
  double cb_p[16], cb_inv[16];    // checkerboard 4x4 plaquettes (row-major)
  std::vector<double> field;      // [t][i] +/-1.0
  Vec G[2];
  Stack left[2], right[2];
  double sign = 1.0, wrap_err = 0.0;
  int64_t accepts = 0;
  std::minstd_rand0 engine;
  const double* inj_u = nullptr;
  size_t inj_n = 0, inj_pos = 0;
  // recorded series (dqmc_walker.cpp:91-92) and equal-time accumulators
  std::vector<Vec> rec[2];
  std::vector<double> rec_sign;
  double acc[ORC_NUM_OBS] = {0};
  int cnt[ORC_NUM_OBS] = {0};
  bool trace_on = false;
  std::vector<Vec> trace;  // pairs (up, dn)
  int kidx = 0;
  // time-displaced Green's functions (dqmc_walker.h:74-80) and G(k, tau) accumulators
  Vec gt0[2], g0t[2];
  std::vector<int> dyn_taus;
  std::vector<double> dyn_sum;
  std::vector<long long> dyn_cnt;
  // density of states, dynamic spin susceptibility and superfluid-stiffness contribution
  // per listed tau (sums over dynamic half-sweeps, sign-weighted as the reference's)
  std::vector<double> dyn_dos, dyn_chi, dyn_rho;
  // per displacement r: sign * 0.5 sum_i (G_up + G_dn)(i + r, i) / N, [tau][r]
  std::vector<double> dyn_r;
  // G(t,t), G(t,0), G(0,t) per spin at the listed tau of the current half-sweep
  std::vector<std::array<Vec, 6>> dyn_rec;

  double& s(int t, int i) { return field[(size_t)t * N + i]; }
  double s(int t, int i) const { return field[(size_t)t * N + i]; }

  void setup(const orc_params& pp) {
    p = pp;
    if (p.L < 1 || (p.lattice != ORC_SQUARE && p.lattice != ORC_CUBIC))
      throw std::invalid_argument("lattice: unknown type or side < 1");
    if (p.lattice == ORC_CUBIC && p.checkerboard)  // dqmc_initializer.cpp:169-182
      throw std::invalid_argument("the checkerboard method is only implemented for the square lattice");
    lat.init(p.L, p.lattice == ORC_CUBIC ? 3 : 2);
    N = lat.N;
    Lt = p.Lt;
    pace = p.pace;
    nstack = (Lt % pace == 0) ? Lt / pace : Lt / pace + 1;
    dtau = p.beta / Lt;
    alpha = std::acosh(std::exp(0.5 * dtau * p.onsite_u));  // repulsive_hubbard.cpp:50
    kidx = p.momentum_index < 0 ? lat.m_point : p.momentum_index;
    // K = -t H + mu I ; expK = exp(-dtau K), inv = exp(+dtau K)  (repulsive_hubbard.cpp:57-68)
    Vec K((size_t)N * N);
    for (size_t k = 0; k < K.size(); ++k) K[k] = -p.hopping_t * lat.hop[k];
    for (int i = 0; i < N; ++i) at(K, N, i, i) += p.mu;
    expK = sym_exp(N, K, -dtau);
    invK = sym_exp(N, K, +dtau);
    transK = transpose(expK, N);
    // checkerboard plaquettes (checkerboard/square.cpp:28-50)
    auto fill = [](double* m, double ch, double sh, double f) {
      const double v[16] = {ch * ch, ch * sh, ch * sh, sh * sh, ch * sh, ch * ch, sh * sh, ch * sh,
                            ch * sh, sh * sh, ch * ch, ch * sh, sh * sh, ch * sh, ch * sh, ch * ch};
      for (int k = 0; k < 16; ++k) m[k] = f * v[k];
    };
    fill(cb_p, std::cosh(dtau * p.hopping_t), std::sinh(dtau * p.hopping_t), std::exp(0.5 * dtau * p.mu));
    fill(cb_inv, std::cosh(-dtau * p.hopping_t), std::sinh(-dtau * p.hopping_t), std::exp(-0.5 * dtau * p.mu));
    field.assign((size_t)Lt * N, 1.0);
    for (int sp = 0; sp < 2; ++sp) {
      G[sp] = identity(N);
      left[sp].init(N, nstack, p.stack_kind);
      right[sp].init(N, nstack, p.stack_kind);
    }
    if (p.record_greens) {
      for (int sp = 0; sp < 2; ++sp) rec[sp].assign(Lt, Vec((size_t)N * N, 0.0));
      rec_sign.assign(Lt, 0.0);
    }
  }

  double uniform() {
    if (inj_u) {
      if (inj_pos >= inj_n) throw std::runtime_error("injected uniform stream exhausted");
      return inj_u[inj_pos++];
    }
    return std::generate_canonical<double, 53>(engine);
  }
  bool bernoulli(double prob) { return uniform() < prob; }  // libstdc++ bernoulli_distribution

  // --- checkerboard (checkerboard/square.cpp:66-226) ------------------------
  void plaq_index(int x, int y, int idx[4]) const {
    const int L = lat.L;
    idx[0] = (x % L) + L * (y % L);
    idx[1] = ((x + 1) % L) + L * (y % L);
    idx[2] = (x % L) + L * ((y + 1) % L);
    idx[3] = ((x + 1) % L) + L * ((y + 1) % L);
  }
  void plaq_left(Vec& m, const double* P, int x, int y) const {
    int idx[4];
    plaq_index(x, y, idx);
    for (int c = 0; c < N; ++c) {
      double v[4], o[4];
      for (int a = 0; a < 4; ++a) v[a] = at(m, N, idx[a], c);
      for (int a = 0; a < 4; ++a) {
        double s2 = 0;
        for (int b = 0; b < 4; ++b) s2 += P[a * 4 + b] * v[b];
        o[a] = s2;
      }
      for (int a = 0; a < 4; ++a) at(m, N, idx[a], c) = o[a];
    }
  }
  void plaq_right(Vec& m, const double* P, int x, int y) const {
    int idx[4];
    plaq_index(x, y, idx);
    for (int r = 0; r < N; ++r) {
      double v[4], o[4];
      for (int a = 0; a < 4; ++a) v[a] = at(m, N, r, idx[a]);
      for (int b = 0; b < 4; ++b) {
        double s2 = 0;
        for (int a = 0; a < 4; ++a) s2 += v[a] * P[a * 4 + b];
        o[b] = s2;
      }
      for (int a = 0; a < 4; ++a) at(m, N, r, idx[a]) = o[a];
    }
  }
  template <class F>
  void layer(int parity, F f) const {
    for (int x = parity; x < lat.L; x += 2)
      for (int y = parity; y < lat.L; y += 2) f(x, y);
  }
  void mult_expK(int which, Vec& m) const {
    if (!p.checkerboard) {  // model_base.cpp:7-35
      switch (which) {
        case 0: m = gemm('N', 'N', N, expK, m); break;
        case 1: m = gemm('N', 'N', N, m, expK); break;
        case 2: m = gemm('N', 'N', N, invK, m); break;
        case 3: m = gemm('N', 'N', N, m, invK); break;
        case 4: m = gemm('N', 'N', N, transK, m); break;
      }
      return;
    }
    const int A = 0, B = 1;  // sublattice A: even corners, B: odd corners
    switch (which) {
      case 0:
        layer(B, [&](int x, int y) { plaq_left(m, cb_p, x, y); });
        layer(A, [&](int x, int y) { plaq_left(m, cb_p, x, y); });
        break;
      case 2:
        layer(A, [&](int x, int y) { plaq_left(m, cb_inv, x, y); });
        layer(B, [&](int x, int y) { plaq_left(m, cb_inv, x, y); });
        break;
      case 1:
        layer(A, [&](int x, int y) { plaq_right(m, cb_p, x, y); });
        layer(B, [&](int x, int y) { plaq_right(m, cb_p, x, y); });
        break;
      case 3:
        layer(B, [&](int x, int y) { plaq_right(m, cb_inv, x, y); });
        layer(A, [&](int x, int y) { plaq_right(m, cb_inv, x, y); });
        break;
      case 4:
        layer(A, [&](int x, int y) { plaq_left(m, cb_p, x, y); });
        layer(B, [&](int x, int y) { plaq_left(m, cb_p, x, y); });
        break;
    }
  }

  // --- B products (repulsive_hubbard.cpp:158-243; attractive uses +1 for spin) ---
  double spin_factor(int spin_sign) const { return p.model == ORC_ATTRACTIVE ? 1.0 : (double)spin_sign; }
  void mult_B(int which, Vec& m, int t, int spin_sign) const {
    const int eff = (t == 0) ? Lt - 1 : t - 1;
    const double sg = spin_factor(spin_sign);
    auto scale_rows = [&](double sgn) {
      for (int i = 0; i < N; ++i) {
        const double e = std::exp(sgn * sg * alpha * s(eff, i));
        for (int c = 0; c < N; ++c) at(m, N, i, c) *= e;
      }
    };
    auto scale_cols = [&](double sgn) {
      for (int i = 0; i < N; ++i) {
        const double e = std::exp(sgn * sg * alpha * s(eff, i));
        for (int r = 0; r < N; ++r) at(m, N, r, i) *= e;
      }
    };
    switch (which) {
      case 0: mult_expK(0, m); scale_rows(+1); break;   // B from left
      case 1: scale_cols(+1); mult_expK(1, m); break;   // B from right
      case 2: scale_rows(-1); mult_expK(2, m); break;   // invB from left
      case 3: mult_expK(3, m); scale_cols(-1); break;   // invB from right
      case 4: scale_rows(+1); mult_expK(4, m); break;   // transB from left
    }
  }

  // --- ratio and rank-1 update -----------------------------------------------
  double update_ratio(int t, int i) const {
    const double si = s(t, i);
    const double gu = at(G[0], N, i, i), gd = at(G[1], N, i, i);
    if (p.model == ORC_REPULSIVE)  // repulsive_hubbard.cpp:112-124
      return (1 + (1 - gu) * (std::exp(-2 * alpha * si) - 1)) * (1 + (1 - gd) * (std::exp(+2 * alpha * si) - 1));
    // attractive_hubbard.cpp:112-125
    return std::exp(2 * alpha * si) * (1 + (1 - gu) * (std::exp(-2 * alpha * si) - 1)) *
           (1 + (1 - gd) * (std::exp(-2 * alpha * si) - 1));
  }
  void rank1(Vec& g, int i, double f) {
    Vec u(N), w(N);
    for (int r = 0; r < N; ++r) u[r] = f * at(g, N, r, i);
    for (int c = 0; c < N; ++c) w[c] = (c == i ? 1.0 : 0.0) - at(g, N, i, c);
    for (int c = 0; c < N; ++c)
      for (int r = 0; r < N; ++r) at(g, N, r, c) -= w[c] * u[r];
  }
  void update_greens(int t, int i) {
    const double si = s(t, i);
    const double gu = at(G[0], N, i, i), gd = at(G[1], N, i, i);
    const double du = std::exp(-2 * alpha * si) - 1;
    const double fu = du / (1 + (1 - gu) * du);
    double fd;
    if (p.model == ORC_REPULSIVE) {  // repulsive_hubbard.cpp:140-147
      const double dd = std::exp(+2 * alpha * si) - 1;
      fd = dd / (1 + (1 - gd) * dd);
    } else {
      fd = fu;  // attractive_hubbard.cpp:149
    }
    rank1(G[0], i, fu);
    rank1(G[1], i, fd);
  }

  // --- walker (dqmc_walker.cpp) -------------------------------------------------
  void init_stacks() {  // :109-134
    Vec tu = identity(N), td = identity(N);
    for (int sp = 0; sp < 2; ++sp) {
      left[sp].len = 0;
      right[sp].len = 0;
    }
    for (int t = Lt; t >= 1; --t) {
      mult_B(4, tu, t, +1);
      mult_B(4, td, t, -1);
      if ((t - 1) % pace == 0) {
        right[0].push(tu);
        right[1].push(td);
        tu = identity(N);
        td = identity(N);
      }
    }
  }
  void init() {
    init_stacks();
    for (int sp = 0; sp < 2; ++sp) G[sp] = equaltime_greens(N, left[sp], right[sp]);  // :137-147
    sign = (det_sign(N, G[0]) * det_sign(N, G[1]) >= 0) ? +1.0 : -1.0;                // :150-163
    wrap_err = 0.0;
  }

  void metropolis(int t) {  // :173-197
    const int eff = (t == 0) ? Lt - 1 : t - 1;
    for (int i = 0; i < N; ++i) {
      const double r = update_ratio(eff, i);
      if (bernoulli(std::min(1.0, std::fabs(r)))) {
        update_greens(eff, i);
        s(eff, i) = -s(eff, i);
        sign = (r >= 0) ? +sign : -sign;
        ++accepts;
      }
    }
  }
  void wrap_fwd(int t) {  // :208-217
    const int eff = (t == Lt) ? 1 : t + 1;
    mult_B(0, G[0], eff, +1);
    mult_B(3, G[0], eff, +1);
    mult_B(0, G[1], eff, -1);
    mult_B(3, G[1], eff, -1);
  }
  void wrap_bwd(int t) {  // :228-237
    const int eff = (t == 0) ? Lt : t;
    mult_B(1, G[0], eff, +1);
    mult_B(2, G[0], eff, +1);
    mult_B(1, G[1], eff, -1);
    mult_B(2, G[1], eff, -1);
  }
  void record(int t) {
    if (!p.record_greens) return;
    rec[0][t - 1] = G[0];
    rec[1][t - 1] = G[1];
    rec_sign[t - 1] = sign;
  }
  void stabilize_common(bool check_error) {
    Vec fresh[2];
    for (int sp = 0; sp < 2; ++sp) fresh[sp] = equaltime_greens(N, left[sp], right[sp]);
    if (check_error) {
      const double e0 = matrix_compare_error(N, fresh[0], G[0]);
      const double e1 = matrix_compare_error(N, fresh[1], G[1]);
      wrap_err = std::max(wrap_err, std::max(e0, e1));
    }
    G[0] = fresh[0];
    G[1] = fresh[1];
    if (trace_on) {
      trace.push_back(G[0]);
      trace.push_back(G[1]);
    }
  }
  void sweep_fwd() {  // :246-325
    Vec tu = identity(N), td = identity(N);
    for (int t = 1; t <= Lt; ++t) {
      wrap_fwd(t - 1);
      metropolis(t);
      record(t);
      mult_B(0, tu, t, +1);
      mult_B(0, td, t, -1);
      if (t % pace == 0 || t == Lt) {
        right[0].pop();
        right[1].pop();
        left[0].push(tu);
        left[1].push(td);
        stabilize_common(true);
        if (p.record_greens) {
          rec[0][t - 1] = G[0];
          rec[1][t - 1] = G[1];
        }
        tu = identity(N);
        td = identity(N);
      }
    }
    if (p.record_greens) {
      rec[0][Lt - 1] = G[0];
      rec[1][Lt - 1] = G[1];
    }
  }
  void sweep_bwd() {  // :334-412
    Vec tu = identity(N), td = identity(N);
    for (int t = Lt; t >= 1; --t) {
      if (t % pace == 0 && t != Lt) {
        left[0].pop();
        left[1].pop();
        right[0].push(tu);
        right[1].push(td);
        stabilize_common(true);
        tu = identity(N);
        td = identity(N);
      }
      metropolis(t);
      record(t);
      mult_B(4, tu, t, +1);
      mult_B(4, td, t, -1);
      wrap_bwd(t);
    }
    left[0].pop();
    left[1].pop();
    right[0].push(tu);
    right[1].push(td);
    stabilize_common(false);
    if (p.record_greens) {
      rec[0][Lt - 1] = G[0];
      rec[1][Lt - 1] = G[1];
    }
  }


  // --- time-displaced Green's functions ------------------------------------------
  // compute_dynamic_greens (numerical_stable.hpp:246-325) for both stack kinds;
  // the stack product is U diag(D) F with F = V^T (SVD) or the QRP right factor.
  void dynamic_greens(int sp, Vec& t0, Vec& ot) const {
    const Stack& L = left[sp];
    const Stack& R = right[sp];
    const Vec I = identity(N);
    if (L.empty()) {  // gt0 = g00, g0t = -(1 - g00)  (:250-257)
      t0 = equaltime_greens(N, L, R);
      ot = t0;
      for (size_t k = 0; k < ot.size(); ++k) ot[k] -= I[k];
      return;
    }
    if (R.empty()) {  // gt0 = (1 + B)^-1 B (compute_greens_b0, :159-179), g0t = -(1 + B)^-1  (:260-270)
      const Level& l = L.top();
      Vec dmax, dmin;
      split_max_min(l.D, dmax, dmin);
      Vec H((size_t)N * N), r1((size_t)N * N), r2((size_t)N * N);
      for (int c = 0; c < N; ++c)
        for (int r = 0; r < N; ++r) {
          const double ut = at(l.U, N, c, r) / dmax[r];  // (Dmax^-1 U^T)(r, c)
          const double vf = dmin[r] * at(l.F, N, r, c);   // (Dmin V^T)(r, c)
          at(H, N, r, c) = ut + vf;
          at(r1, N, r, c) = vf;
          at(r2, N, r, c) = ut;
        }
      if (L.kind == ORC_STACK_SVD) {  // the reference's fullPivHouseholderQr solves
        t0 = fullpiv_qr_solve(N, H, r1);
        ot = fullpiv_qr_solve(N, H, r2);
      } else {
        std::vector<int> piv;
        int ns;
        lu_factor(N, H, piv, ns);
        lu_solve(N, H, piv, r1, N);
        lu_solve(N, H, piv, r2, N);
        t0 = r1;
        ot = r2;
      }
      for (auto& x : ot) x = -x;
      return;
    }
    const Level& l = L.top();
    const Level& r = R.top();
    Vec dlmax, dlmin, drmax, drmin;
    split_max_min(l.D, dlmax, dlmin);
    split_max_min(r.D, drmax, drmin);
    // gt0 = U_R Drmax^-1 [Dlmax^-1 U_L^T U_R Drmax^-1 + Dlmin V_L^T V_R Drmin]^-1 Dlmin V_L^T
    {
      const Vec A = gemm('T', 'N', N, l.U, r.U);
      const Vec B = gemm('N', 'T', N, l.F, r.F);
      Vec M((size_t)N * N), rhs((size_t)N * N);
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          at(M, N, i, j) = at(A, N, i, j) / (dlmax[i] * drmax[j]) + at(B, N, i, j) * dlmin[i] * drmin[j];
          at(rhs, N, i, j) = dlmin[i] * at(l.F, N, i, j);
        }
      std::vector<int> piv;
      int ns;
      lu_factor(N, M, piv, ns);
      lu_solve(N, M, piv, rhs, N);
      Vec ur = r.U;
      for (int c = 0; c < N; ++c)
        for (int i = 0; i < N; ++i) at(ur, N, i, c) /= drmax[c];
      t0 = gemm('N', 'N', N, ur, rhs);
    }
    if (L.kind != ORC_STACK_SVD) {
      // the right factors of the QRP stack are not orthogonal, so the reference's
      // second formula does not apply; by push-through, (1 + B_R B_L)^-1 B_R =
      // B_R (1 + B_L B_R)^-1 with B_R = F_R^T D_R U_R^T gives
      // g0t = -F_R^T Drmin M^-1 Dlmax^-1 U_L^T (the M of the equal-time form)
      const Vec A = gemm('T', 'N', N, l.U, r.U);
      const Vec B = gemm('N', 'T', N, l.F, r.F);
      Vec M((size_t)N * N), rhs((size_t)N * N);
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          at(M, N, i, j) = at(A, N, i, j) / (dlmax[i] * drmax[j]) + at(B, N, i, j) * dlmin[i] * drmin[j];
          at(rhs, N, i, j) = at(l.U, N, j, i) / dlmax[i];
        }
      std::vector<int> piv;
      int ns;
      lu_factor(N, M, piv, ns);
      lu_solve(N, M, piv, rhs, N);
      Vec frt = transpose(r.F, N);
      for (int c = 0; c < N; ++c)
        for (int i = 0; i < N; ++i) at(frt, N, i, c) *= -drmin[c];
      ot = gemm('N', 'N', N, frt, rhs);
      return;
    }
    // g0t = -V_L Dlmax^-1 [Drmax^-1 V_R^T V_L Dlmax^-1 + Drmin U_R^T U_L Dlmin]^-1 Drmin U_R^T
    {
      const Vec X = gemm('N', 'T', N, r.F, l.F);
      const Vec Y = gemm('T', 'N', N, r.U, l.U);
      Vec M((size_t)N * N), rhs((size_t)N * N);
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          at(M, N, i, j) = at(X, N, i, j) / (drmax[i] * dlmax[j]) + at(Y, N, i, j) * drmin[i] * dlmin[j];
          at(rhs, N, i, j) = drmin[i] * at(r.U, N, j, i);
        }
      std::vector<int> piv;
      int ns;
      lu_factor(N, M, piv, ns);
      lu_solve(N, M, piv, rhs, N);
      Vec vl = transpose(l.F, N);
      for (int c = 0; c < N; ++c)
        for (int i = 0; i < N; ++i) at(vl, N, i, c) /= -dlmax[c];
      ot = gemm('N', 'N', N, vl, rhs);
    }
  }
  // measure_greens_functions (measure_methods.cpp:278-308) at one tau for this walker's momentum
  void accumulate_dynamic(int slot, const Vec& gu, const Vec& gd) {
    double sum = 0.0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        sum += sign * 0.5 * (at(gu, N, j, i) + at(gd, N, j, i)) / N * lat.fourier(lat.disp(i, j), kidx);
    dyn_sum[slot] += sum;
    dyn_cnt[slot] += 1;
    for (int r = 0; r < N; ++r) {
      double sr = 0.0;
      for (int i = 0; i < N; ++i) {
        const int j = lat.shift(i, r);  // disp(i, j) = r
        sr += sign * 0.5 * (at(gu, N, j, i) + at(gd, N, j, i)) / N;
      }
      dyn_r[(size_t)slot * N + r] += sr;
    }
  }
  // The dynamic observables of measure_methods.cpp:315-461 for the listed tau, from the
  // recorded G(t,t), G(t,0), G(0,t) (tau >= 1: slice tau; tau = 0: the reference's
  // index Lt-1, i.e. G(beta,beta), G(beta,0), G(0,beta)) and g00 = G(beta,beta):
  //   density of states (316-332): sign tr(G(t,0) spin-averaged) / N, G(beta,beta) at tau = 0;
  //   dynamic spin susceptibility (422-461): 0.25 sign / N sum_i (Gc(t,t)_ii Gc00_ii - G(0,t)_ii G(t,0)_ii
  //     for both spins - Gc(t,t)up_ii Gc00dn_ii - Gc00up_ii Gc(t,t)dn_ii), Gc = I - G^T;
  //   superfluid stiffness (345-416): 0.25 t^2 sign / N^2 sum_ij (cos kx rx - cos kx ry) (uncorrelated
  //     and correlated current terms), one contribution per tau (the reference sums them over all tau).
  void measure_dynamic_obs(int ntau) {
    const double s = sign, invN = 1.0 / N, kx1 = lat.nk > 1 ? lat.kx[1] : 0.0;
    const Vec& g00u = G[0];
    const Vec& g00d = G[1];
    for (int k = 0; k < ntau; ++k) {
      const int t = dyn_taus[k];
      const auto& r = dyn_rec[k];
      const Vec &gttu = r[0], &gttd = r[1], &gt0u = r[2], &gt0d = r[3], &g0tu = r[4], &g0td = r[5];
      // density of states: G(beta,beta) at tau = 0 (the reference's Greentt(Lt-1))
      const Vec& du = (t == 0) ? gttu : gt0u;
      const Vec& dd = (t == 0) ? gttd : gt0d;
      double tr = 0.0;
      for (int i = 0; i < N; ++i) tr += 0.5 * (at(du, N, i, i) + at(dd, N, i, i));
      dyn_dos[k] += s * tr * invN;
      double chi = 0.0;
      for (int i = 0; i < N; ++i) {
        const double gcttu = 1.0 - at(gttu, N, i, i), gcttd = 1.0 - at(gttd, N, i, i);
        const double gc00u = 1.0 - at(g00u, N, i, i), gc00d = 1.0 - at(g00d, N, i, i);
        chi += 0.25 * s * invN *
               (+gcttu * gc00u - at(g0tu, N, i, i) * at(gt0u, N, i, i) + gcttd * gc00d -
                at(g0td, N, i, i) * at(gt0d, N, i, i) - gcttu * gc00d - gc00u * gcttd);
      }
      dyn_chi[k] += chi;
      // the superfluid stiffness is a square-lattice observable (dqmc_initializer.cpp:233-237
      // drops it elsewhere; measure_methods.cpp:350 asserts the square lattice)
      if (lat.dim != 2) continue;
      double rho = 0.0;
      for (int i = 0; i < N; ++i) {
        const int ipx = lat.nn[i * 4 + 0];
        for (int j = 0; j < N; ++j) {
          const int jpx = lat.nn[j * 4 + 0];
          const int d = lat.disp(i, j), rx = d % lat.L, ry = d / lat.L;
          const double ff = std::cos(-rx * kx1) - std::cos(-ry * kx1);  // FourierFactor(rx,1) - (ry,1)
          rho += p.hopping_t * p.hopping_t * s * ff *
                 (-(at(gttu, N, j, jpx) - at(gttu, N, jpx, j) + at(gttd, N, j, jpx) - at(gttd, N, jpx, j)) *
                      (at(g00u, N, i, ipx) - at(g00u, N, ipx, i) + at(g00d, N, i, ipx) - at(g00d, N, ipx, i)) -
                  at(g0tu, N, ipx, jpx) * at(gt0u, N, j, i) - at(g0td, N, ipx, jpx) * at(gt0d, N, j, i) +
                  at(g0tu, N, i, jpx) * at(gt0u, N, j, ipx) + at(g0td, N, i, jpx) * at(gt0d, N, j, ipx) +
                  at(g0tu, N, ipx, j) * at(gt0u, N, jpx, i) + at(g0td, N, ipx, j) * at(gt0d, N, jpx, i) -
                  at(g0tu, N, i, j) * at(gt0u, N, jpx, ipx) - at(g0td, N, i, j) * at(gt0d, N, jpx, ipx));
        }
      }
      dyn_rho[k] += 0.25 * rho / ((double)N * N);
    }
  }
  // sweep_for_dynamic_greens (dqmc_walker.cpp:424-524): 0 -> beta with the fields fixed
  void sweep_dynamic(const int* taus, int ntau) {
    if (!left[0].empty() || right[0].len != nstack)
      throw std::runtime_error("sweep_dynamic: needs the stacks of t = 0 (after init or a backward sweep)");
    if ((int)dyn_taus.size() != ntau || !std::equal(dyn_taus.begin(), dyn_taus.end(), taus)) {
      dyn_taus.assign(taus, taus + ntau);
      dyn_sum.assign(ntau, 0.0);
      dyn_cnt.assign(ntau, 0);
      dyn_dos.assign(ntau, 0.0);
      dyn_chi.assign(ntau, 0.0);
      dyn_rho.assign(ntau, 0.0);
      dyn_r.assign((size_t)ntau * N, 0.0);
    }
    dyn_rec.assign(ntau, {});
    const Vec I = identity(N);
    for (int sp = 0; sp < 2; ++sp) {
      gt0[sp] = G[sp];
      g0t[sp] = G[sp];
      for (size_t k = 0; k < g0t[sp].size(); ++k) g0t[sp][k] -= I[k];
    }
    Vec tu = identity(N), td = identity(N);
    for (int t = 1; t <= Lt; ++t) {
      wrap_fwd(t - 1);
      mult_B(0, gt0[0], t, +1);
      mult_B(0, gt0[1], t, -1);
      mult_B(3, g0t[0], t, +1);
      mult_B(3, g0t[1], t, -1);
      mult_B(0, tu, t, +1);
      mult_B(0, td, t, -1);
      if (t % pace == 0 || t == Lt) {
        right[0].pop();
        right[1].pop();
        left[0].push(tu);
        left[1].push(td);
        for (int sp = 0; sp < 2; ++sp) {
          G[sp] = equaltime_greens(N, left[sp], right[sp]);
          Vec f0, f1;
          dynamic_greens(sp, f0, f1);
          wrap_err = std::max(wrap_err, std::max(matrix_compare_error(N, f0, gt0[sp]), matrix_compare_error(N, f1, g0t[sp])));
          gt0[sp] = f0;
          g0t[sp] = f1;
        }
        if (trace_on) {
          trace.push_back(gt0[0]);
          trace.push_back(gt0[1]);
        }
        tu = identity(N);
        td = identity(N);
      }
      for (int k = 0; k < ntau; ++k)
        if (taus[k] == t && t < Lt) {
          accumulate_dynamic(k, gt0[0], gt0[1]);
          dyn_rec[k] = {G[0], G[1], gt0[0], gt0[1], g0t[0], g0t[1]};
        }
    }
    for (int k = 0; k < ntau; ++k)
      if (taus[k] == 0) {
        accumulate_dynamic(k, G[0], G[1]);  // tau = 0: G(beta, beta) = G(0, 0)
        dyn_rec[k] = {G[0], G[1], gt0[0], gt0[1], g0t[0], g0t[1]};  // index Lt-1: t = beta
      }
    measure_dynamic_obs(ntau);
    dyn_rec.clear();
  }

  // --- equal-time measurements (measure_methods.cpp:22-255) ---------------------
  void measure() {
    if (!p.record_greens) throw std::runtime_error("measure() needs record_greens");
    const double invN = 1.0 / N;
    for (int t = 0; t < Lt; ++t) {
      const Vec& gu = rec[0][t];
      const Vec& gd = rec[1][t];
      const double sg = rec_sign[t];
      acc[ORC_OBS_SIGN] += sg;
      cnt[ORC_OBS_SIGN] += 1;
      double tr = 0, dbl = 0, kin = 0, loc = 0;
      for (int i = 0; i < N; ++i) {
        const double a = at(gu, N, i, i), b = at(gd, N, i, i);
        tr += a + b;
        dbl += (1 - a) * (1 - b);
        loc += sg * (a + b - 2 * a * b);
        for (int dir = 0; dir < lat.dim; ++dir) {  // +x, +y (, +z): measure_methods.cpp:87-95
          const int j = lat.nn[i * 2 * lat.dim + dir];
          kin += at(gu, N, i, j) + at(gd, N, i, j);
        }
      }
      acc[ORC_OBS_FILLING] += sg * (2 - tr / N);
      acc[ORC_OBS_DOUBLE_OCC] += sg * dbl / N;
      acc[ORC_OBS_KINETIC] += sg * (2 * p.hopping_t) * kin / N;
      acc[ORC_OBS_LOCAL_SPIN] += loc / N;
      double nk = 0, sdw = 0, cdw = 0, sw = 0;
      for (int i = 0; i < N; ++i) {
        const double guc_ii = 1 - at(gu, N, i, i), gdc_ii = 1 - at(gd, N, i, i);
        for (int j = 0; j < N; ++j) {
          const double ff = lat.fourier(lat.disp(i, j), kidx);
          const double guc_jj = 1 - at(gu, N, j, j), gdc_jj = 1 - at(gd, N, j, j);
          const double guc_ij = (i == j ? 1.0 : 0.0) - at(gu, N, j, i);
          const double gdc_ij = (i == j ? 1.0 : 0.0) - at(gd, N, j, i);
          nk += (at(gu, N, j, i) + at(gd, N, j, i)) * ff;
          const double common = guc_ii * guc_jj + guc_ij * at(gu, N, i, j) + gdc_ii * gdc_jj + gdc_ij * at(gd, N, i, j);
          sdw += sg * ff * (common - gdc_ii * guc_jj - guc_ii * gdc_jj);
          cdw += sg * ff * (common + gdc_ii * guc_jj + guc_ii * gdc_jj);
          sw += sg * (guc_ij * gdc_ij);
        }
      }
      acc[ORC_OBS_MOMENTUM_DIST] += sg * (1 - 0.5 * nk / N);
      acc[ORC_OBS_SDW] += sdw / ((double)N * N);
      acc[ORC_OBS_CDW] += cdw / ((double)N * N);
      acc[ORC_OBS_SWAVE] += sw / N;
      for (int k = 0; k < 8; ++k) cnt[k] += 1;
    }
    (void)invN;
  }
  void write_bin(double* out) {  // measure_handler.cpp:170-240
    const double sgn = acc[ORC_OBS_SIGN] / cnt[ORC_OBS_SIGN];
    for (int k = 0; k < 8; ++k) out[k] = acc[k] / (cnt[k] * sgn);
    out[ORC_OBS_SIGN] = std::fabs(sgn);
    for (int k = 0; k < ORC_NUM_OBS; ++k) { acc[k] = 0; cnt[k] = 0; }
  }
};

Oracle* O(void* h) { return static_cast<Oracle*>(h); }

}  // namespace

// ============================================================================
// C interface
// ============================================================================
extern "C" {

void orc_set_lapack(orc_dgemm_t gemm_fn, orc_dgesvd_t gesvd_fn) {
  g_dgemm = gemm_fn;
  g_dgesvd = gesvd_fn;
}

void* orc_create(const orc_params* p) {
  auto* o = new Oracle();
  try {
    o->setup(*p);
  } catch (const std::exception&) {
    delete o;
    return nullptr;
  }
  return o;
}
void orc_destroy(void* h) { delete O(h); }
int orc_space_size(void* h) { return O(h)->N; }
void orc_seed(void* h, unsigned seed) { O(h)->engine.seed(seed); }
double orc_draw_uniform(void* h) { return std::generate_canonical<double, 53>(O(h)->engine); }
void orc_set_uniforms(void* h, const double* u, size_t n) {
  O(h)->inj_u = u;
  O(h)->inj_n = n;
  O(h)->inj_pos = 0;
}

void orc_fields_random(void* h) {
  Oracle* o = O(h);
  for (int t = 0; t < o->Lt; ++t)
    for (int i = 0; i < o->N; ++i) o->s(t, i) = o->bernoulli(0.5) ? +1.0 : -1.0;
}
void orc_set_fields(void* h, const int8_t* f) {
  Oracle* o = O(h);
  for (size_t k = 0; k < o->field.size(); ++k) o->field[k] = f[k] > 0 ? 1.0 : -1.0;
}
void orc_get_fields(void* h, int8_t* f) {
  Oracle* o = O(h);
  for (size_t k = 0; k < o->field.size(); ++k) f[k] = o->field[k] > 0 ? 1 : -1;
}
void orc_init(void* h) { O(h)->init(); }
void orc_sweep_0_to_beta(void* h) { O(h)->sweep_fwd(); }
void orc_sweep_beta_to_0(void* h) { O(h)->sweep_bwd(); }
void orc_measure(void* h) { O(h)->measure(); }
int orc_sweep_dynamic(void* h, const int* taus, int ntau) {
  try {
    O(h)->sweep_dynamic(taus, ntau);
  } catch (const std::exception&) {
    return -1;
  }
  return 0;
}
void orc_get_dynamic(void* h, double* sums, int64_t* counts) {
  for (size_t k = 0; k < O(h)->dyn_sum.size(); ++k) {
    sums[k] = O(h)->dyn_sum[k];
    counts[k] = O(h)->dyn_cnt[k];
  }
}
void orc_get_dynamic_r(void* h, double* out) {
  std::copy(O(h)->dyn_r.begin(), O(h)->dyn_r.end(), out);
}
void orc_get_dynamic_obs(void* h, double* dos, double* chi, double* rho) {
  for (size_t k = 0; k < O(h)->dyn_dos.size(); ++k) {
    dos[k] = O(h)->dyn_dos[k];
    chi[k] = O(h)->dyn_chi[k];
    rho[k] = O(h)->dyn_rho[k];
  }
}
void orc_get_green_dynamic(void* h, int which, int spin, double* out) {
  const Vec& g = which == 0 ? O(h)->gt0[spin] : O(h)->g0t[spin];
  std::memcpy(out, g.data(), sizeof(double) * g.size());
}
void orc_write_bin(void* h, int, double* out) { O(h)->write_bin(out); }
void orc_get_accumulators(void* h, double* sums, int* counts) {
  for (int k = 0; k < ORC_NUM_OBS; ++k) {
    sums[k] = O(h)->acc[k];
    counts[k] = O(h)->cnt[k];
  }
}
void orc_get_green(void* h, int spin, double* out) {
  std::memcpy(out, O(h)->G[spin].data(), sizeof(double) * O(h)->G[spin].size());
}
void orc_set_green(void* h, int spin, const double* in) {
  std::memcpy(O(h)->G[spin].data(), in, sizeof(double) * O(h)->G[spin].size());
}
double orc_wrap_error(void* h) { return O(h)->wrap_err; }
double orc_config_sign(void* h) { return O(h)->sign; }
void orc_set_config_sign(void* h, double s) { O(h)->sign = (s >= 0) ? 1.0 : -1.0; }
int64_t orc_accept_count(void* h) { return O(h)->accepts; }
int orc_trace_count(void* h) { return (int)O(h)->trace.size() / 2; }
void orc_trace_get(void* h, int k, int spin, double* out) {
  const Vec& g = O(h)->trace[(size_t)2 * k + spin];
  std::memcpy(out, g.data(), sizeof(double) * g.size());
}
void orc_trace_clear(void* h) { O(h)->trace.clear(); }
void orc_trace_enable(void* h, int on) { O(h)->trace_on = on != 0; }

double orc_update_ratio(void* h, int eff_t, int i) { return O(h)->update_ratio(eff_t, i); }
void orc_update_greens(void* h, int eff_t, int i) { O(h)->update_greens(eff_t, i); }
void orc_mult_B(void* h, int which, double* mat, int t, int spin) {
  Oracle* o = O(h);
  Vec m(mat, mat + (size_t)o->N * o->N);
  o->mult_B(which, m, t, spin);
  std::memcpy(mat, m.data(), sizeof(double) * m.size());
}
void orc_mult_expK(void* h, int which, double* mat) {
  Oracle* o = O(h);
  Vec m(mat, mat + (size_t)o->N * o->N);
  o->mult_expK(which, m);
  std::memcpy(mat, m.data(), sizeof(double) * m.size());
}
void orc_get_expK(void* h, int which, double* out) {
  Oracle* o = O(h);
  const Vec& m = which == 0 ? o->expK : which == 1 ? o->invK : o->lat.hop;
  std::memcpy(out, m.data(), sizeof(double) * m.size());
}
double orc_alpha(void* h) { return O(h)->alpha; }

void orc_svd(int n, const double* a, double* u, double* s, double* v) {
  Vec A(a, a + (size_t)n * n), U, S, V;
  svd(n, A, U, S, V);
  std::memcpy(u, U.data(), sizeof(double) * U.size());
  std::memcpy(s, S.data(), sizeof(double) * S.size());
  std::memcpy(v, V.data(), sizeof(double) * V.size());
}
void orc_qrp_udt(int n, const double* a, double* u, double* d, double* t) {
  Vec A(a, a + (size_t)n * n), U, D, T;
  qrp_udt(n, A, U, D, T);
  std::memcpy(u, U.data(), sizeof(double) * U.size());
  std::memcpy(d, D.data(), sizeof(double) * D.size());
  std::memcpy(t, T.data(), sizeof(double) * T.size());
}
void orc_greens_from_udv(int n, const double* u, const double* d, const double* f, double* g) {
  Vec U(u, u + (size_t)n * n), D(d, d + n), F(f, f + (size_t)n * n);
  Vec G = greens_udf(n, U, D, F);
  std::memcpy(g, G.data(), sizeof(double) * G.size());
}

int orc_num_k_stars(void* h) { return O(h)->lat.nk; }
int orc_m_point_index(void* h) { return O(h)->lat.m_point; }
double orc_fourier_factor(void* h, int disp, int k) { return O(h)->lat.fourier(disp, k); }
int orc_space_dim(void* h) { return O(h)->lat.dim; }
int orc_nearest_neighbour(void* h, int i, int dir) { return O(h)->lat.nn[(size_t)i * 2 * O(h)->lat.dim + dir]; }
int orc_displacement(void* h, int i, int j) { return O(h)->lat.disp(i, j); }
void orc_k_star(void* h, int k, double* out) {
  const Lattice& l = O(h)->lat;
  out[0] = l.kx[k];
  out[1] = l.ky[k];
  if (l.dim == 3) out[2] = l.kz[k];
}

}  // extern "C"
