// Compile-time operator tables: for each Green block, the (out p, in q, sign)
// pairs that use it, for the N / N^H / K / K^H operators in the PWC (C=3) and
// PWL (C=12) bases.  Built at compile time from the reference's tables
// (pq: mvp_N_pwc_tucker.m:12, mvp_K_pwc_tucker.m:12; llp: mvp_N_pwl_tucker.m:13;
// slp: mvp_N_herm_adj_pwl_tucker.m:14) so that the z-pass multiply can loop
// over blocks with every index a constant after unrolling.
#pragma once

namespace marie {

struct OpEntry {
  int blk, p, q, sgn;
};

template <int NE>
struct OpList {
  OpEntry e[NE];
  int s1[60], s2[60], s3[60];   // circulant mirror signs per block
  int nblk;
};

constexpr int ct_abs(int v) { return v < 0 ? -v : v; }
constexpr int ct_sgn(int v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

// op: 0 N, 1 N^H, 2 K, 3 K^H
constexpr int op_entries(bool pwl, int op) {
  const bool isK = op >= 2;
  const int pairs = isK ? 6 : 9;
  return pairs * (pwl ? 16 : 1);
}

template <bool PWL, int OP>
constexpr OpList<op_entries(PWL, OP)> make_oplist() {
  constexpr int PQ_N[3][3] = {{1, 2, 3}, {2, 4, 5}, {3, 5, 6}};
  constexpr int PQ_K[3][3] = {{0, -3, 2}, {3, 0, -1}, {-2, 1, 0}};
  constexpr int LLP[4][4] = {{1, 5, 6, 7}, {-5, 2, 8, 9}, {-6, 8, 3, 10}, {-7, 9, 10, 4}};
  constexpr int SLP[4][4] = {{1, -1, -1, -1}, {-1, 1, 1, 1}, {-1, 1, 1, 1}, {-1, 1, 1, 1}};
  constexpr int GN[3][6] = {{+1, -1, -1, +1, +1, +1}, {+1, -1, +1, +1, -1, +1}, {+1, +1, -1, +1, -1, +1}};
  constexpr int GK[3][3] = {{-1, +1, +1}, {+1, -1, +1}, {+1, +1, -1}};
  constexpr int BT[3][10] = {{+1, +1, +1, +1, -1, +1, +1, -1, -1, +1},
                             {+1, +1, +1, +1, +1, -1, +1, -1, +1, -1},
                             {+1, +1, +1, +1, +1, +1, -1, +1, -1, -1}};
  constexpr bool isK = OP >= 2, adj = (OP & 1) != 0;
  constexpr int ncomp = isK ? 3 : 6;
  constexpr int pwx = PWL ? 10 : 1;
  OpList<op_entries(PWL, OP)> L{};
  L.nblk = pwx * ncomp;
  for (int j = 0; j < 60; ++j) { L.s1[j] = 1; L.s2[j] = 1; L.s3[j] = 1; }
  for (int j = 0; j < pwx; ++j)
    for (int k = 0; k < ncomp; ++k) {
      const int id = j * ncomp + k;
      L.s1[id] = (isK ? GK[0][k] : GN[0][k]) * (PWL ? BT[0][j] : 1);
      L.s2[id] = (isK ? GK[1][k] : GN[1][k]) * (PWL ? BT[1][j] : 1);
      L.s3[id] = (isK ? GK[2][k] : GN[2][k]) * (PWL ? BT[2][j] : 1);
    }
  int n = 0;
  // entries ordered by block so that each block's value is loaded once
  for (int blk = 0; blk < pwx * ncomp; ++blk) {
    for (int P = 0; P < 3; ++P) {
      for (int Q = 0; Q < 3; ++Q) {
        const bool skip = isK && P == Q;
        const int k = isK ? ct_abs(PQ_K[P][Q]) - 1 : PQ_N[P][Q] - 1;
        const int spq = isK ? ct_sgn(PQ_K[P][Q]) : 1;
        if (!skip && !PWL && k == blk) {
          L.e[n] = OpEntry{blk, P, Q, (isK && adj) ? -spq : spq};
          ++n;
        }
        if (!skip && PWL) {
          for (int l = 0; l < 4; ++l) {
            for (int lp = 0; lp < 4; ++lp) {
              const int j = ct_abs(LLP[l][lp]) - 1;
              if (j * ncomp + k == blk) {
                int s = spq * ct_sgn(LLP[l][lp]);
                if (adj) s *= ct_sgn(SLP[l][lp]) * (isK ? -1 : 1);
                L.e[n] = OpEntry{blk, 4 * P + l, 4 * Q + lp, s};
                ++n;
              }
            }
          }
        }
      }
    }
  }
  return L;
}

template <bool PWL, int OP>
struct OpTab {
  static constexpr auto L = make_oplist<PWL, OP>();
  static constexpr int NE = op_entries(PWL, OP);
};

}  // namespace marie
