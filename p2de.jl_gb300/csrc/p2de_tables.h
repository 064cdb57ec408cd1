// Operator tables for tensor-product GLL quads, one per N1D = N+1 in 2..6, built on
// the host from the 1D GLL rule the way initialize_operators (src/dg/init.jl:133-228)
// builds the dense operators, then reduced to the entries that are nonzero for LGL:
//   Srh_db/Ssh_db volume blocks (Qr - Qr', init.jl:152-155) along r- and s-lines,
//   Sr0/Ss0 (init.jl:312-322) on r- and s-neighbours,
//   wq and 1/wq (the diagonal of M \ Vh', init.jl:171),
// plus the pair lists and per-node gather orders that reproduce the accumulation
// order of the nnz loops of init.jl:188-204.
#pragma once

#include <stdint.h>

namespace p2de {

constexpr int kMaxN1D = 6;
// the table of log_fast: F_j = j / 256 for j = kLogTabLo .. kLogTabLo + kLogTabN - 1, which
// covers the reduced mantissas [sqrt(1/2), sqrt(2)) to the nearest 1/256
constexpr int kLogTabLo = 181;
constexpr int kLogTabN = 182;
constexpr int kMaxNq = kMaxN1D * kMaxN1D;
constexpr int kMaxPairsHi = kMaxN1D * kMaxN1D * (kMaxN1D - 1);  // 180
constexpr int kMaxPairsLo = 2 * kMaxN1D * (kMaxN1D - 1);        // 60

struct OpTable {
  int32_t N1D, Nq, Nfp, npl, nph;
  int32_t basis;  // p2de_basis: 0 LGL nodes, 1 Gauss nodes
  double w1D[kMaxN1D];
  double wq[kMaxNq];
  double rwq[kMaxNq];  // 1.0 / wq
  // high-order volume pairs (i > j), r-lines first then s-lines
  int16_t hp_i[kMaxPairsHi];
  int16_t hp_j[kMaxPairsHi];
  int8_t hp_axis[kMaxPairsHi];  // 0: r-line (Srh_db), 1: s-line (Ssh_db)
  double hp_S[kMaxPairsHi];     // Srh_db[i,j] or Ssh_db[i,j]
  // per-node gather list, partners in ascending node index: pair id, +1 when the node is i
  int16_t hg_pair[kMaxNq][2 * (kMaxN1D - 1)];
  int8_t hg_sign[kMaxNq][2 * (kMaxN1D - 1)];
  // low-order pairs (i > j): r-neighbours first then s-neighbours
  int16_t lp_i[kMaxPairsLo];
  int16_t lp_j[kMaxPairsLo];
  int8_t lp_axis[kMaxPairsLo];
  double lp_S[kMaxPairsLo];  // Sr0[i,j] or Ss0[i,j]
  int16_t lg_pair[kMaxNq][4];
  int8_t lg_sign[kMaxNq][4];
  int8_t lg_count[kMaxNq];
  int8_t hg_count[kMaxNq];
  // FP32 copies for the mixed-precision high-order terms
  float hp_Sf[kMaxPairsHi];
  float rwqf[kMaxNq];
  // the gather lists split by axis (r-line partners, s-line partners), each in the
  // merged lists' order; used where a pair contributes to its own axis only
  int16_t hga_pair[2][kMaxNq][kMaxN1D - 1];
  int8_t hga_sign[2][kMaxNq][kMaxN1D - 1];
  int16_t lga_pair[2][kMaxNq][2];
  int8_t lga_sign[2][kMaxNq][2];
  int8_t lga_count[2][kMaxNq];
  // inv(VDM) of the orthonormal Legendre products P_i(r) P_j(s), mode i + N1D j (init.jl:224),
  // row-major Nq x Nq: the modal coefficients of nodal values (HennemannShockCapture)
  double VDMinv[kMaxNq * kMaxNq];
  // Gauss nodes: the Lagrange basis at r = -1 and r = +1, the face extrapolation Vf
  // along a line (construct_gauss_reference_data, init.jl:111-131); LGL: unit vectors
  double ellm[kMaxN1D];
  double ellp[kMaxN1D];
  // the lift M \ Vf' of the unlimited projection at node m from its four faces (sides
  // r=-1, r=+1, s=-1, s=+1 in order): Vf[f, m] / wq[m] (init.jl:171-172)
  double liftf[kMaxNq][4];
  // log_fast: per j, 1/F_j, log F_j to 41 significant bits and the rest of log F_j; log 2 in
  // the same two parts (42 significant bits, so that k log2_hi is exact for |k| < 2048)
  double logtab[kLogTabN][3];
  double ln2_hi, ln2_lo;
};

// Builds the table for polynomial degree N (1..5) on the LGL (basis 0) or Gauss (basis 1)
// nodes. Returns 0 on success.
int build_op_table(int N, double zerotol, OpTable* out, int basis = 0);

// Operators of a Line element (initialize_reference_data(::Dim1), init.jl:66-80, with
// initialize_operators, :133-228): N1D nodes, face nodes r = -1 (0) and r = +1 (1).
constexpr int kLineMaxNh = kMaxN1D + 2;
constexpr int kLineMaxPairs = kLineMaxNh * (kLineMaxNh - 1) / 2;
struct LineOps {
  int32_t N1D, basis, npair;
  double wq[kMaxN1D];
  double rxf[2];                          // Br: -1, +1 (nrJ with wf = 1)
  double Vf[2][kMaxN1D];                  // face extrapolation (LGL: unit vectors)
  double Sh[kLineMaxNh * kLineMaxNh];     // Srh_db = [Q - Q', Ef' B; -B Ef, 0], column-major Nh x Nh
  int8_t pi[kLineMaxPairs], pj[kLineMaxPairs];  // its nonzero pairs i > j, j outer (init.jl:188-195)
  double MinvVhT[kMaxN1D * kLineMaxNh];   // M \ Vh' = (1/wq) [I, Vf'], column-major Nq x Nh
  double VDMinv[kMaxN1D * kMaxN1D];       // inv(VDM) of the orthonormal Legendre modes, row-major
};

// Builds the Line operators for degree N (1..5) on LGL (basis 0) or Gauss (basis 1) nodes.
int build_line_ops(int N, double zerotol, LineOps* out, int basis);

// The 1D Gauss-Legendre rule (nodes, weights), differentiation matrix (row-major) and the
// Lagrange basis at -1 and +1.
void gauss_rule(int N, double* r, double* w, double* D, double* ellm, double* ellp);

// The 1D GLL rule (nodes, weights) and differentiation matrix (row-major).
void gll_rule(int N, double* r, double* w, double* D);

}  // namespace p2de
