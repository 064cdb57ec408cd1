// Host construction of the GLL operator tables (see p2de_tables.h).
#include "p2de_tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace p2de {

// GLL nodes by Newton iteration on (1-x^2)P_N'(x) written with the Legendre
// recurrence (Hesthaven & Warburton, Nodal Discontinuous Galerkin Methods, 2008,
// sec. 3.2), weights 2/(N(N+1)P_N(x_i)^2), and the Lagrange differentiation matrix
// D_ij = P_N(x_i)/(P_N(x_j)(x_i - x_j)), D_00 = -N(N+1)/4, D_NN = N(N+1)/4.
void gll_rule(int N, double* r, double* w, double* D) {
  const int Np = N + 1;
  std::vector<double> x(Np), xold(Np), P(Np * (N + 1));
  for (int i = 0; i < Np; ++i) x[i] = -std::cos(M_PI * i / N);
  auto legendre = [&]() {
    for (int i = 0; i < Np; ++i) {
      double* Pi = &P[i * (N + 1)];
      Pi[0] = 1.0;
      if (N >= 1) Pi[1] = x[i];
      for (int k = 2; k <= N; ++k) Pi[k] = ((2.0 * k - 1.0) * x[i] * Pi[k - 1] - (k - 1.0) * Pi[k - 2]) / k;
    }
  };
  for (int it = 0; it < 100; ++it) {
    xold = x;
    legendre();
    double err = 0.0;
    for (int i = 0; i < Np; ++i) {
      const double* Pi = &P[i * (N + 1)];
      x[i] = xold[i] - (x[i] * Pi[N] - Pi[N - 1]) / (Np * Pi[N]);
      err = std::max(err, std::fabs(x[i] - xold[i]));
    }
    if (err < 1e-16) break;
  }
  for (int i = 0; i < Np / 2; ++i) {
    double a = 0.5 * (x[Np - 1 - i] - x[i]);
    x[i] = -a;
    x[Np - 1 - i] = a;
  }
  if (Np % 2 == 1) x[Np / 2] = 0.0;
  x[0] = -1.0;
  x[Np - 1] = 1.0;
  legendre();
  for (int i = 0; i < Np; ++i) {
    double PN = P[i * (N + 1) + N];
    r[i] = x[i];
    w[i] = 2.0 / (N * Np * PN * PN);
  }
  for (int i = 0; i < Np; ++i)
    for (int j = 0; j < Np; ++j) {
      double v;
      if (i != j)
        v = P[i * (N + 1) + N] / (P[j * (N + 1) + N] * (x[i] - x[j]));
      else if (i == 0)
        v = -N * (N + 1) / 4.0;
      else if (i == N)
        v = N * (N + 1) / 4.0;
      else
        v = 0.0;
      D[i * Np + j] = v;
    }
}

// Gauss-Legendre nodes: the roots of P_{N+1} by Newton iteration from
// x_i = -cos(pi (i + 3/4) / (N + 3/2)), weights 2 / ((1 - x^2) P'_{N+1}(x)^2); the
// Lagrange basis in barycentric form (Berrut & Trefethen, SIAM Review 46, 2004):
// D_ij = (l_j / l_i) / (x_i - x_j), D_ii = -sum_j D_ij, values at -1 and +1 from the
// second barycentric formula.
void gauss_rule(int N, double* r, double* w, double* D, double* ellm, double* ellp) {
  const int n = N + 1;
  auto legendre = [&](double x, double& P, double& dP) {  // P_n(x) and P_n'(x)
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; ++k) {
      const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    P = p1;
    dP = n * (x * p1 - p0) / (x * x - 1.0);
  };
  for (int i = 0; i < n; ++i) {
    double x = -std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double P, dP;
      legendre(x, P, dP);
      const double dx = P / dP;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    r[i] = x;
  }
  for (int i = 0; i < n / 2; ++i) {
    const double a = 0.5 * (r[n - 1 - i] - r[i]);
    r[i] = -a;
    r[n - 1 - i] = a;
  }
  if (n % 2 == 1) r[n / 2] = 0.0;
  for (int i = 0; i < n; ++i) {
    double P, dP;
    legendre(r[i], P, dP);
    w[i] = 2.0 / ((1.0 - r[i] * r[i]) * dP * dP);
  }
  double lam[kMaxN1D];
  for (int j = 0; j < n; ++j) {
    lam[j] = 1.0;
    for (int k = 0; k < n; ++k)
      if (k != j) lam[j] /= (r[j] - r[k]);
  }
  for (int i = 0; i < n; ++i) {
    double diag = 0.0;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        D[i * n + j] = (lam[j] / lam[i]) / (r[i] - r[j]);
        diag -= D[i * n + j];
      }
    D[i * n + i] = diag;
  }
  for (int side = 0; side < 2; ++side) {
    const double x = side == 0 ? -1.0 : 1.0;
    double den = 0.0;
    for (int j = 0; j < n; ++j) den += lam[j] / (x - r[j]);
    for (int j = 0; j < n; ++j) (side == 0 ? ellm : ellp)[j] = (lam[j] / (x - r[j])) / den;
  }
}

namespace {

// Legendre polynomial of degree n normalized on [-1, 1] (three-term recurrence)
double legendre_normalized(int n, double x) {
  if (n == 0) return std::sqrt(0.5);
  double p0 = 1.0, p1 = x;
  for (int k = 1; k < n; ++k) {
    const double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
    p0 = p1;
    p1 = p2;
  }
  return std::sqrt((2.0 * n + 1.0) / 2.0) * p1;
}

// inverse of a small dense matrix (row-major m x m) by Gauss-Jordan with partial pivoting
bool invert(std::vector<double> A, int m, double* inv) {
  std::vector<double> I((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) I[(size_t)i * m + i] = 1.0;
  for (int c = 0; c < m; ++c) {
    int piv = c;
    for (int r = c + 1; r < m; ++r)
      if (std::fabs(A[(size_t)r * m + c]) > std::fabs(A[(size_t)piv * m + c])) piv = r;
    if (A[(size_t)piv * m + c] == 0.0) return false;
    if (piv != c)
      for (int j = 0; j < m; ++j) {
        std::swap(A[(size_t)c * m + j], A[(size_t)piv * m + j]);
        std::swap(I[(size_t)c * m + j], I[(size_t)piv * m + j]);
      }
    const double d = A[(size_t)c * m + c];
    for (int j = 0; j < m; ++j) {
      A[(size_t)c * m + j] /= d;
      I[(size_t)c * m + j] /= d;
    }
    for (int r = 0; r < m; ++r) {
      if (r == c) continue;
      const double f = A[(size_t)r * m + c];
      if (f == 0.0) continue;
      for (int j = 0; j < m; ++j) {
        A[(size_t)r * m + j] -= f * A[(size_t)c * m + j];
        I[(size_t)r * m + j] -= f * I[(size_t)c * m + j];
      }
    }
  }
  for (size_t i = 0; i < I.size(); ++i) inv[i] = I[i];
  return true;
}

}  // namespace

// The table of log_fast (in the stage kernels): a value rounded to double and cut to its
// leading `bits` significant bits, and the rest.
static void split_hi_lo(long double v, int bits, double* hi, double* lo) {
  double h = (double)v;
  uint64_t b;
  std::memcpy(&b, &h, sizeof b);
  b &= ~((1ull << (52 - (bits - 1))) - 1);
  std::memcpy(&h, &b, sizeof b);
  *hi = h;
  *lo = (double)(v - (long double)h);
}

int build_op_table(int N, double zerotol, OpTable* T, int basis) {
  if (N < 1 || N + 1 > kMaxN1D || basis < 0 || basis > 1) return 1;
  std::memset(T, 0, sizeof(OpTable));
  for (int i = 0; i < kLogTabN; ++i) {
    const int j = kLogTabLo + i;
    T->logtab[i][0] = 256.0 / j;
    split_hi_lo(std::log((long double)j / 256.0L), 41, &T->logtab[i][1], &T->logtab[i][2]);
  }
  split_hi_lo(std::log(2.0L), 42, &T->ln2_hi, &T->ln2_lo);
  const int n = N + 1, Nq = n * n;
  T->N1D = n;
  T->Nq = Nq;
  T->Nfp = 4 * n;
  T->basis = basis;
  double r[kMaxN1D], w[kMaxN1D], D[kMaxN1D * kMaxN1D];
  if (basis == 1) {
    gauss_rule(N, r, w, D, T->ellm, T->ellp);
    for (int a = 0; a < n; ++a) {  // droptol'd like Vf (init.jl:140-143)
      if (std::fabs(T->ellm[a]) <= zerotol) T->ellm[a] = 0.0;
      if (std::fabs(T->ellp[a]) <= zerotol) T->ellp[a] = 0.0;
    }
  } else {
    gll_rule(N, r, w, D);
    T->ellm[0] = 1.0;
    T->ellp[N] = 1.0;
  }
  for (int is = 0; is < n; ++is)
    for (int ir = 0; ir < n; ++ir) {
      const double wqm = w[ir] * w[is];
      const int m = ir + n * is;
      T->liftf[m][0] = T->ellm[ir] / wqm;
      T->liftf[m][1] = T->ellp[ir] / wqm;
      T->liftf[m][2] = T->ellm[is] / wqm;
      T->liftf[m][3] = T->ellp[is] / wqm;
    }
  for (int i = 0; i < n; ++i) T->w1D[i] = w[i];
  // node i = ir + n*is; wq = wr .* ws
  for (int is = 0; is < n; ++is)
    for (int ir = 0; ir < n; ++ir) {
      T->wq[ir + n * is] = w[ir] * w[is];
      T->rwq[ir + n * is] = 1.0 / (w[ir] * w[is]);
    }
  // Qr = diag(wq) * kron(I, D1D), Qs = diag(wq) * kron(D1D, I), droptol'd
  std::vector<double> Qr(Nq * Nq, 0.0), Qs(Nq * Nq, 0.0);  // row-major [i][j]
  for (int is = 0; is < n; ++is)
    for (int ir = 0; ir < n; ++ir)
      for (int jr = 0; jr < n; ++jr) {
        int i = ir + n * is, j = jr + n * is;
        double q = T->wq[i] * D[ir * n + jr];
        Qr[i * Nq + j] = std::fabs(q) <= zerotol ? 0.0 : q;
      }
  for (int ir = 0; ir < n; ++ir)
    for (int is = 0; is < n; ++is)
      for (int js = 0; js < n; ++js) {
        int i = ir + n * is, j = ir + n * js;
        double q = T->wq[i] * D[is * n + js];
        Qs[i * Nq + j] = std::fabs(q) <= zerotol ? 0.0 : q;
      }
  // high-order pairs in the volume block of Srsh_db = Q - Q'
  int p = 0;
  for (int is = 0; is < n; ++is)
    for (int ir = 1; ir < n; ++ir)
      for (int jr = 0; jr < ir; ++jr) {
        int i = ir + n * is, j = jr + n * is;
        T->hp_i[p] = (int16_t)i;
        T->hp_j[p] = (int16_t)j;
        T->hp_axis[p] = 0;
        T->hp_S[p] = Qr[i * Nq + j] - Qr[j * Nq + i];
        ++p;
      }
  for (int ir = 0; ir < n; ++ir)
    for (int is = 1; is < n; ++is)
      for (int js = 0; js < is; ++js) {
        int i = ir + n * is, j = ir + n * js;
        T->hp_i[p] = (int16_t)i;
        T->hp_j[p] = (int16_t)j;
        T->hp_axis[p] = 1;
        T->hp_S[p] = Qs[i * Nq + j] - Qs[j * Nq + i];
        ++p;
      }
  T->nph = p;
  {
    std::vector<double> V((size_t)Nq * Nq);
    for (int is = 0; is < n; ++is)
      for (int ir = 0; ir < n; ++ir)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i)
            V[(size_t)(ir + n * is) * Nq + (i + n * j)] = legendre_normalized(i, r[ir]) * legendre_normalized(j, r[is]);
    if (!invert(V, Nq, T->VDMinv)) return 4;
  }
  for (int q = 0; q < p; ++q) T->hp_Sf[q] = (float)T->hp_S[q];
  for (int m = 0; m < Nq; ++m) T->rwqf[m] = (float)T->rwq[m];
  // gather order per node: partners ascending (the order in which the j-outer,
  // i-inner nnz loop of init.jl:188-195 touches the node)
  for (int m = 0; m < Nq; ++m) {
    std::vector<std::pair<int, int>> lst;  // (partner, pair id)
    for (int q = 0; q < p; ++q) {
      if (T->hp_i[q] == m) lst.push_back({T->hp_j[q], q});
      if (T->hp_j[q] == m) lst.push_back({T->hp_i[q], q});
    }
    std::sort(lst.begin(), lst.end());
    T->hg_count[m] = (int8_t)lst.size();
    int na[2] = {0, 0};
    for (size_t t = 0; t < lst.size(); ++t) {
      const int q = lst[t].second;
      T->hg_pair[m][t] = (int16_t)q;
      T->hg_sign[m][t] = (T->hp_i[q] == m) ? 1 : -1;
      const int ax = T->hp_axis[q];
      if (na[ax] >= n - 1) return 3;
      T->hga_pair[ax][m][na[ax]] = (int16_t)q;
      T->hga_sign[ax][m][na[ax]] = T->hg_sign[m][t];
      ++na[ax];
    }
    if (na[0] != n - 1 || na[1] != n - 1) return 3;
  }
  // low order: Q01D tridiagonal (init.jl:276-295), Qr0 = kron(M1D, Q01D), Qs0 = kron(Q01D, M1D)
  std::vector<double> Q01(n * n, 0.0);  // row-major
  for (int i = 0; i + 1 < n; ++i) {
    Q01[(i + 1) * n + i] = -0.5;
    Q01[i * n + (i + 1)] = 0.5;
  }
  Q01[0] = -0.5;
  Q01[(n - 1) * n + (n - 1)] = 0.5;
  // Qr0 = droptol!(kron(M1D, Q01D)), Qs0 = droptol!(kron(Q01D, M1D)), and Sr0, Ss0 =
  // droptol!(0.5 (Q0 - Q0')) (low_order_operators, init.jl:312-321)
  auto drop = [&](double v) { return std::fabs(v) <= zerotol ? 0.0 : v; };
  auto Qr0 = [&](int i, int j) {
    int ir = i % n, is = i / n, jr = j % n, js = j / n;
    return drop((is == js ? w[is] : 0.0) * Q01[ir * n + jr]);
  };
  auto Qs0 = [&](int i, int j) {
    int ir = i % n, is = i / n, jr = j % n, js = j / n;
    return drop(Q01[is * n + js] * (ir == jr ? w[ir] : 0.0));
  };
  p = 0;
  for (int is = 0; is < n; ++is)
    for (int ir = 0; ir + 1 < n; ++ir) {
      int i = (ir + 1) + n * is, j = ir + n * is;
      T->lp_i[p] = (int16_t)i;
      T->lp_j[p] = (int16_t)j;
      T->lp_axis[p] = 0;
      T->lp_S[p] = drop(0.5 * (Qr0(i, j) - Qr0(j, i)));
      ++p;
    }
  for (int ir = 0; ir < n; ++ir)
    for (int is = 0; is + 1 < n; ++is) {
      int i = ir + n * (is + 1), j = ir + n * is;
      T->lp_i[p] = (int16_t)i;
      T->lp_j[p] = (int16_t)j;
      T->lp_axis[p] = 1;
      T->lp_S[p] = drop(0.5 * (Qs0(i, j) - Qs0(j, i)));
      ++p;
    }
  T->npl = p;
  for (int m = 0; m < Nq; ++m) {
    std::vector<std::pair<int, int>> lst;
    for (int q = 0; q < p; ++q) {
      if (T->lp_i[q] == m) lst.push_back({T->lp_j[q], q});
      if (T->lp_j[q] == m) lst.push_back({T->lp_i[q], q});
    }
    std::sort(lst.begin(), lst.end());
    T->lg_count[m] = (int8_t)lst.size();
    for (size_t t = 0; t < lst.size(); ++t) {
      const int q = lst[t].second;
      T->lg_pair[m][t] = (int16_t)q;
      T->lg_sign[m][t] = (T->lp_i[q] == m) ? 1 : -1;
      const int ax = T->lp_axis[q];
      const int c = T->lga_count[ax][m];
      if (c >= 2) return 3;
      T->lga_pair[ax][m][c] = (int16_t)q;
      T->lga_sign[ax][m][c] = T->lg_sign[m][t];
      T->lga_count[ax][m] = (int8_t)(c + 1);
    }
  }
  return 0;
}

}  // namespace p2de

namespace p2de {

int build_line_ops(int N, double zerotol, LineOps* T, int basis) {
  if (N < 1 || N + 1 > kMaxN1D || basis < 0 || basis > 1) return 1;
  std::memset(T, 0, sizeof(LineOps));
  const int n = N + 1, Nh = n + 2;
  double r[kMaxN1D], w[kMaxN1D], D[kMaxN1D * kMaxN1D], ellm[kMaxN1D], ellp[kMaxN1D];
  if (basis == 1) {
    gauss_rule(N, r, w, D, ellm, ellp);
  } else {
    gll_rule(N, r, w, D);
    for (int i = 0; i < n; ++i) ellm[i] = ellp[i] = 0.0;
    ellm[0] = 1.0;
    ellp[N] = 1.0;
  }
  T->N1D = n;
  T->basis = basis;
  T->rxf[0] = -1.0;
  T->rxf[1] = 1.0;
  for (int i = 0; i < n; ++i) {
    T->wq[i] = w[i];
    T->Vf[0][i] = std::fabs(ellm[i]) <= zerotol ? 0.0 : ellm[i];
    T->Vf[1][i] = std::fabs(ellp[i]) <= zerotol ? 0.0 : ellp[i];
  }
  // Q = M Dr with droptol! (init.jl:149); Srh_db of the hybridized operator (init.jl:150-155)
  std::vector<double> Q((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double q = w[i] * D[i * n + j];
      Q[i + (size_t)n * j] = std::fabs(q) <= zerotol ? 0.0 : q;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) T->Sh[i + Nh * j] = Q[i + (size_t)n * j] - Q[j + (size_t)n * i];
  for (int f = 0; f < 2; ++f)
    for (int i = 0; i < n; ++i) {
      const double e = T->Vf[f][i];
      if (e == 0.0) continue;
      T->Sh[i + Nh * (n + f)] = e * T->rxf[f];
      T->Sh[(n + f) + Nh * i] = -(T->rxf[f] * e);
    }
  if (basis == 1)
    for (int i = 0; i < Nh * Nh; ++i)
      if (std::fabs(0.5 * T->Sh[i]) <= zerotol) T->Sh[i] = 0.0;
  int np = 0;
  for (int j = 0; j < Nh; ++j)
    for (int i = j + 1; i < Nh; ++i)
      if (T->Sh[i + Nh * j] != 0.0) {
        T->pi[np] = (int8_t)i;
        T->pj[np] = (int8_t)j;
        ++np;
      }
  T->npair = np;
  for (int i = 0; i < n; ++i) {
    T->MinvVhT[i + n * i] = 1.0 / w[i];
    for (int f = 0; f < 2; ++f)
      if (T->Vf[f][i] != 0.0) T->MinvVhT[i + n * (n + f)] = T->Vf[f][i] / w[i];
  }
  std::vector<double> V((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[(size_t)i * n + j] = legendre_normalized(j, r[i]);
  return invert(V, n, T->VDMinv) ? 0 : 2;
}

}  // namespace p2de
