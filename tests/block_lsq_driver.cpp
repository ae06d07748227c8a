// Host test driver of blocklsq.h: reads p, m, S0 (p x p) and the block
// Hessenberg matrix Hbar ((m+1)p x mp, column-major complex128) from a binary
// file, runs the block least-squares updates step by step and writes the
// residual norms of every step, the final Y and Z, and a Cholesky check.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "blocklsq.h"

using marie::zc;

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int hdr[2];
  if (std::fread(hdr, sizeof(int), 2, f) != 2) return 4;
  const int p = hdr[0], m = hdr[1], ld = (m + 1) * p;
  std::vector<zc> S0((size_t)p * p), H((size_t)ld * m * p), A((size_t)p * p);
  if (std::fread(S0.data(), sizeof(zc), S0.size(), f) != S0.size()) return 5;
  if (std::fread(H.data(), sizeof(zc), H.size(), f) != H.size()) return 6;
  if (std::fread(A.data(), sizeof(zc), A.size(), f) != A.size()) return 7;
  std::fclose(f);
  marie::BlockLsq lsq;
  lsq.init(p, m, S0);
  std::vector<double> res_all, resid;
  for (int j = 0; j < m; ++j) {
    const int rows = (j + 2) * p;
    std::vector<zc> Hc((size_t)rows * p);
    for (int c = 0; c < p; ++c)
      for (int i = 0; i < rows; ++i) Hc[i + (size_t)rows * c] = H[i + (size_t)ld * (j * p + c)];
    lsq.add_block(j, Hc, resid);
    res_all.insert(res_all.end(), resid.begin(), resid.end());
  }
  std::vector<zc> Y, Z, R, Ri;
  lsq.solve(m - 1, Y);
  lsq.residual(m - 1, Z);
  const bool ok = marie::cholesky_upper(A, p, 0.0, R);
  marie::tri_inverse(R, p, Ri);
  const std::vector<zc> I = marie::tri_mul(R, Ri, p);
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 8;
  std::fwrite(res_all.data(), sizeof(double), res_all.size(), g);
  std::fwrite(Y.data(), sizeof(zc), Y.size(), g);
  std::fwrite(Z.data(), sizeof(zc), Z.size(), g);
  const int okv = ok ? 1 : 0;
  std::fwrite(&okv, sizeof(int), 1, g);
  std::fwrite(R.data(), sizeof(zc), R.size(), g);
  std::fwrite(I.data(), sizeof(zc), I.size(), g);
  std::fclose(g);
  return 0;
}
