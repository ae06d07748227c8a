// Host-side dense algebra of the block GMRES solver (bgmres.cuh), in FP64:
// Cholesky QR factors of p x p Gram matrices and the least-squares problem
// min_Y || [S; 0] - Hbar Y ||_F of the block Hessenberg matrix by Householder
// reflections.  Plain C++ (no CUDA), so that it also builds into the host
// test of tests/test_block_lsq.py.
#pragma once
#include <cmath>
#include <complex>
#include <cstdint>
#include <thread>
#include <vector>

namespace marie {

typedef std::complex<double> zc;

// Run f(i) for i in [0, n) on up to 16 host threads.
template <typename F>
static void parallel_for(int n, int64_t work, F f) {
  const int hw = (int)std::thread::hardware_concurrency();
  const int nt = work < 2000000 ? 1 : std::min(n, std::max(1, std::min(hw, 16)));
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (int i = t; i < n; i += nt) f(i);
    });
  for (auto& x : th) x.join();
}

// Upper Cholesky A = R^H R of a Hermitian p x p matrix (column-major) with a
// diagonal shift; false if a pivot is not positive.
static bool cholesky_upper(const std::vector<zc>& A, int p, double shift, std::vector<zc>& R) {
  R.assign((size_t)p * p, zc(0, 0));
  for (int j = 0; j < p; ++j) {
    for (int i = 0; i <= j; ++i) {
      zc s = A[i + (size_t)p * j];
      if (i == j) s += shift;
      for (int k = 0; k < i; ++k) s -= std::conj(R[k + (size_t)p * i]) * R[k + (size_t)p * j];
      if (i == j) {
        if (!(s.real() > 0) || !std::isfinite(s.real())) return false;
        R[j + (size_t)p * j] = zc(std::sqrt(s.real()), 0);
      } else {
        R[i + (size_t)p * j] = s / R[i + (size_t)p * i].real();
      }
    }
  }
  return true;
}

// inverse of an upper-triangular p x p matrix (column-major)
static void tri_inverse(const std::vector<zc>& R, int p, std::vector<zc>& Ri) {
  Ri.assign((size_t)p * p, zc(0, 0));
  for (int j = 0; j < p; ++j) {
    Ri[j + (size_t)p * j] = 1.0 / R[j + (size_t)p * j];
    for (int i = j - 1; i >= 0; --i) {
      zc s = 0;
      for (int k = i + 1; k <= j; ++k) s += R[i + (size_t)p * k] * Ri[k + (size_t)p * j];
      Ri[i + (size_t)p * j] = -s / R[i + (size_t)p * i];
    }
  }
}

// C = A B for upper-triangular p x p matrices
static std::vector<zc> tri_mul(const std::vector<zc>& A, const std::vector<zc>& B, int p) {
  std::vector<zc> C((size_t)p * p, zc(0, 0));
  for (int j = 0; j < p; ++j)
    for (int i = 0; i <= j; ++i) {
      zc s = 0;
      for (int k = i; k <= j; ++k) s += A[i + (size_t)p * k] * B[k + (size_t)p * j];
      C[i + (size_t)p * j] = s;
    }
  return C;
}

// Householder QR of the block Hessenberg matrix, column block by column block.
struct BlockLsq {
  int p = 0, m = 0, ld = 0;        // block size, block steps, rows (m+1)p
  std::vector<zc> Rt;              // transformed Hbar, ld x mp
  std::vector<zc> Vh;              // reflector of column q: p+1 entries (rows q..q+p)
  std::vector<double> coef;        // 2 / (v^H v), 0 for the identity
  std::vector<zc> G;               // transformed right-hand side, ld x p
  void init(int p_, int m_, const std::vector<zc>& S0) {
    p = p_;
    m = m_;
    ld = (m + 1) * p;
    Rt.assign((size_t)ld * m * p, zc(0, 0));
    Vh.assign((size_t)m * p * (p + 1), zc(0, 0));
    coef.assign((size_t)m * p, 0.0);
    G.assign((size_t)ld * p, zc(0, 0));
    for (int c = 0; c < p; ++c)
      for (int i = 0; i < p; ++i) G[i + (size_t)ld * c] = S0[i + (size_t)p * c];
  }
  // y (rows q..q+p of a column with stride 1) -= coef v (v^H y)
  void reflect(int q, zc* y) const {
    const double cf = coef[q];
    if (cf == 0.0) return;
    const zc* v = &Vh[(size_t)q * (p + 1)];
    zc s = 0;
    for (int i = 0; i <= p; ++i) s += std::conj(v[i]) * y[i];
    s *= cf;
    for (int i = 0; i <= p; ++i) y[i] -= s * v[i];
  }
  // Hc: (j+2)p x p, column-major with leading dimension (j+2)p: block column j
  // of Hbar.  Returns the residual norm of every column after step j.
  void add_block(int j, const std::vector<zc>& Hc, std::vector<double>& resid) {
    const int rows = (j + 2) * p;
    zc* R = &Rt[(size_t)ld * j * p];
    for (int c = 0; c < p; ++c)
      for (int i = 0; i < rows; ++i) R[i + (size_t)ld * c] = Hc[i + (size_t)rows * c];
    // earlier reflectors, column by column (independent)
    parallel_for(p, (int64_t)j * p * p * p * 8, [&](int c) {
      zc* col = R + (size_t)ld * c;
      for (int q = 0; q < j * p; ++q) reflect(q, col + q);
    });
    // new reflectors: column q = jp + c zeroes rows q+1..q+p
    for (int c = 0; c < p; ++c) {
      const int q = j * p + c;
      zc* x = R + (size_t)ld * c + q;
      double tail = 0;
      for (int i = 1; i <= p; ++i) tail += std::norm(x[i]);
      zc* v = &Vh[(size_t)q * (p + 1)];
      if (tail == 0.0) {
        coef[q] = 0.0;
        for (int i = 0; i <= p; ++i) v[i] = 0;
        continue;
      }
      const double nx = std::sqrt(std::norm(x[0]) + tail);
      const double ax = std::abs(x[0]);
      const zc ph = ax > 0 ? x[0] / ax : zc(1, 0);
      const zc alpha = -ph * nx;
      v[0] = x[0] - alpha;
      for (int i = 1; i <= p; ++i) v[i] = x[i];
      const double vn = std::norm(v[0]) + tail;
      coef[q] = 2.0 / vn;
      x[0] = alpha;
      for (int i = 1; i <= p; ++i) x[i] = 0;
      for (int c2 = c + 1; c2 < p; ++c2) reflect(q, R + (size_t)ld * c2 + q);
      for (int c2 = 0; c2 < p; ++c2) reflect(q, &G[(size_t)ld * c2 + q]);
    }
    resid.assign(p, 0.0);
    for (int c = 0; c < p; ++c) {
      double s = 0;
      for (int i = (j + 1) * p; i < (j + 2) * p; ++i) s += std::norm(G[i + (size_t)ld * c]);
      resid[c] = std::sqrt(s);
    }
  }
  // Y ((j+1)p x p) = Rt^{-1} G_top after step j
  void solve(int j, std::vector<zc>& Y) const {
    const int n = (j + 1) * p;
    Y.assign((size_t)n * p, zc(0, 0));
    parallel_for(p, (int64_t)n * n * p * 4, [&](int c) {
      zc* y = &Y[(size_t)n * c];
      for (int i = n - 1; i >= 0; --i) {
        zc s = G[i + (size_t)ld * c];
        for (int k = i + 1; k < n; ++k) s -= Rt[i + (size_t)ld * k] * y[k];
        const zc d = Rt[i + (size_t)ld * i];
        y[i] = std::abs(d) > 0 ? s / d : zc(0, 0);
      }
    });
  }
  // Z ((j+2)p x p) = Q [0; G_bottom]: the residual block in the basis V_{0:j+1}
  void residual(int j, std::vector<zc>& Z) const {
    const int n = (j + 2) * p;
    Z.assign((size_t)n * p, zc(0, 0));
    parallel_for(p, (int64_t)n * p * p * 8, [&](int c) {
      zc* z = &Z[(size_t)n * c];
      for (int i = (j + 1) * p; i < n; ++i) z[i] = G[i + (size_t)ld * c];
      for (int q = (j + 1) * p - 1; q >= 0; --q) reflect(q, z + q);
    });
  }
};

}  // namespace marie
