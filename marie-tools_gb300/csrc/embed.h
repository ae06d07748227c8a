// Grid embedding: operator data of an n1 x n2 x n3 grid restated on a larger
// m1 x m2 x m3 grid, so that grids whose edges have a prime factor above 31
// (which the FFT passes do not cover) still run, and grids with all edges
// <= 128 can take the four-step passes (edges 16*NB).
//
// Why this is exact: mvp_N is a linear convolution of the grid currents with
// the Green's tensor over offsets -(n-1)..(n-1) per axis, evaluated through a
// circulant of size 2n (assembly_fft_circ_tucker_{pwc,pwl}.m).  Any circulant
// of size 2m >= 2n - 1 gives the same convolution on the caller's grid,
// provided the Green's tensor is zero at the offsets n..m-1 it never had.  So
// the caller's voxel (i, j, k) becomes (i, j, k) of the larger grid, the
// voxels added at the high end of each axis hold no body (they are absent
// from idx_solution), and the operator is the caller's, zero-padded:
//  * dense I_V (n1, n2, n3, pwx, ncomp): copied into (m1, m2, m3, pwx, ncomp);
//  * Tucker factors U = FFT_2n(ext), ext = [u(0..n-1), 0, s u(n-1..1)] per
//    rank row: ext is recovered by an inverse DFT of length 2n and moved to
//    the extension of length 2m with the same entries at offsets
//    -(n-1)..(n-1) (so the mirror sign s needs no table), then transformed
//    by a DFT of length 2m; the core G is unchanged.
// Body vectors keep their layout (idx_solution order), so mvp_vie, GMRES and
// the field maps see no difference; operators on full grids would see the
// larger grid and are refused on such handles.
//
// Host-only C++ (no CUDA): the creation path calls it before any upload.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/marie_gb300.h"

namespace marie {
namespace embed {

// All prime factors <= 31: the FFT lengths the passes are built for (for
// edges <= 1024 this is exactly what the FFT plan accepts).
inline bool smooth31(int n) {
  if (n < 1) return false;
  for (int p = 2; p <= 31; ++p)
    while (n % p == 0) n /= p;
  return n == 1;
}

// Grid the caller's n is embedded in; false when it runs as given.
//  * some edge not 31-smooth, or `force`: every edge <= 128 -> all edges
//    rounded up to multiples of 16 (the four-step passes need all three);
//    otherwise each non-smooth edge -> the next 31-smooth length;
//  * nothing to do (all smooth and not forced, or already 16*NB) -> false.
inline bool embed_dims(const int n[3], bool force, int m[3]) {
  bool need = false, small = true;
  for (int d = 0; d < 3; ++d) {
    m[d] = n[d];
    if (!smooth31(n[d])) need = true;
    if (n[d] > 128) small = false;
  }
  if (!need && !force) return false;
  for (int d = 0; d < 3; ++d) {
    if (small) {
      m[d] = (n[d] + 15) / 16 * 16;
    } else {
      int v = n[d];
      while (!smooth31(v)) ++v;
      m[d] = v;
    }
  }
  return m[0] != n[0] || m[1] != n[1] || m[2] != n[2];
}

// Caller's 0-based linear voxel index -> index on the embedded grid.
inline int64_t remap_voxel(int64_t lin, const int n[3], const int m[3]) {
  const int64_t i = lin % n[0];
  const int64_t j = (lin / n[0]) % n[1];
  const int64_t k = lin / ((int64_t)n[0] * n[1]);
  return i + (int64_t)m[0] * (j + (int64_t)m[1] * k);
}

// Interleaved-complex array of nblk column-major (n1, n2, n3) blocks copied
// into zero-filled (m1, m2, m3) blocks; `fill` is the value of added voxels.
inline void pad_grid(const double* src, const int n[3], const int m[3], int64_t nblk, double fill_re,
                     std::vector<double>& dst) {
  const int64_t mD = (int64_t)m[0] * m[1] * m[2];
  dst.assign((size_t)(2 * mD * nblk), 0.0);
  if (fill_re != 0.0)
    for (int64_t q = 0; q < mD * nblk; ++q) dst[2 * q] = fill_re;
  for (int64_t b = 0; b < nblk; ++b)
    for (int64_t k = 0; k < n[2]; ++k)
      for (int64_t j = 0; j < n[1]; ++j) {
        const int64_t s = ((b * n[2] + k) * n[1] + j) * n[0];
        const int64_t t = ((b * m[2] + k) * m[1] + j) * m[0];
        std::memcpy(&dst[2 * t], &src[2 * s], sizeof(double) * 2 * n[0]);
      }
}

// One Tucker factor U (r x 2n, column-major, interleaved complex) restated
// for an axis of length m >= n: U' (r x 2m).
inline void embed_factor(const double* U, int r, int n, int m, std::vector<double>& out) {
  using cd = std::complex<double>;
  const int L = 2 * n, Lm = 2 * m;
  const long double pi = 3.141592653589793238462643383279502884L;
  std::vector<cd> wi(L), wf(Lm);
  for (int q = 0; q < L; ++q) {
    const long double a = 2.0L * pi * (long double)q / (long double)L;
    wi[q] = cd((double)std::cos(a), (double)std::sin(a));     // e^{+2 pi i q / L}
  }
  for (int q = 0; q < Lm; ++q) {
    const long double a = -2.0L * pi * (long double)q / (long double)Lm;
    wf[q] = cd((double)std::cos(a), (double)std::sin(a));     // e^{-2 pi i q / Lm}
  }
  out.assign((size_t)2 * r * Lm, 0.0);
  std::vector<cd> ext(L);
  std::vector<int> pos;   // positions on the 2m extension of ext's entries (x != n)
  std::vector<int> from;
  for (int x = 0; x < n; ++x) { from.push_back(x); pos.push_back(x); }
  for (int jj = 1; jj < n; ++jj) { from.push_back(L - jj); pos.push_back(Lm - jj); }
  for (int rho = 0; rho < r; ++rho) {
    for (int x = 0; x < L; ++x) {
      if (x == n) { ext[x] = 0.0; continue; }
      cd acc = 0.0;
      for (int k = 0; k < L; ++k) {
        const cd u(U[2 * (rho + (int64_t)r * k)], U[2 * (rho + (int64_t)r * k) + 1]);
        acc += u * wi[(int)(((int64_t)k * x) % L)];
      }
      ext[x] = acc / (double)L;
    }
    for (int k = 0; k < Lm; ++k) {
      cd acc = 0.0;
      for (size_t e = 0; e < pos.size(); ++e) acc += ext[from[e]] * wf[(int)(((int64_t)k * pos[e]) % Lm)];
      out[2 * (rho + (int64_t)r * k)] = acc.real();
      out[2 * (rho + (int64_t)r * k) + 1] = acc.imag();
    }
  }
}

// Host copies behind an embedded descriptor (they must outlive creation).
struct Buffers {
  std::vector<int64_t> idx;
  std::vector<double> mr, denseN, denseK;
  std::vector<marie_tucker_block> tkN, tkK;
  std::vector<std::vector<double>> factors;
};

inline void embed_tucker(const marie_tucker_block* tk, int nblk, const int n[3], const int m[3], Buffers& buf,
                         std::vector<marie_tucker_block>& out) {
  out.assign(tk, tk + nblk);
  for (int b = 0; b < nblk; ++b) {
    marie_tucker_block& t = out[b];
    if (t.r1 < 1 || t.r2 < 1 || t.r3 < 1 || !t.U1 || !t.U2 || !t.U3) continue;   // rejected at upload
    const double* U[3] = {t.U1, t.U2, t.U3};
    const int r[3] = {t.r1, t.r2, t.r3};
    for (int d = 0; d < 3; ++d) {
      if (m[d] == n[d]) continue;
      buf.factors.emplace_back();
      embed_factor(U[d], r[d], n[d], m[d], buf.factors.back());
      U[d] = buf.factors.back().data();
    }
    t.U1 = U[0];
    t.U2 = U[1];
    t.U3 = U[2];
  }
}

// The descriptor `e` of the embedded grid m for the caller's descriptor `d`
// (already validated: idx_solution component-major and inside the grid).
inline void embed_desc(const marie_vie_desc* d, const int m[3], Buffers& buf, marie_vie_desc* e) {
  const int n[3] = {d->n1, d->n2, d->n3};
  const int C = d->basis == MARIE_PWL ? 12 : 3;
  const int pwx = d->basis == MARIE_PWL ? 10 : 1;
  const int64_t Ns = d->n_b / C;
  const int64_t mD = (int64_t)m[0] * m[1] * m[2];
  *e = *d;
  e->n1 = m[0];
  e->n2 = m[1];
  e->n3 = m[2];
  buf.factors.reserve(3 * 60 * 2);   // pointers into it are kept: no reallocation
  buf.idx.resize((size_t)d->n_b);
  for (int64_t s = 0; s < Ns; ++s) {
    const int64_t v = remap_voxel(d->idx_solution[s], n, m);
    for (int c = 0; c < C; ++c) buf.idx[(size_t)(c * Ns + s)] = c * mD + v;
  }
  e->idx_solution = buf.idx.data();
  pad_grid(d->Mr, n, m, 1, 1.0, buf.mr);   // Mr = 1 (air) on the added voxels
  e->Mr = buf.mr.data();
  if (d->tucker_N) {
    embed_tucker(d->tucker_N, pwx * 6, n, m, buf, buf.tkN);
    e->tucker_N = buf.tkN.data();
  } else if (d->dense_N) {
    pad_grid(d->dense_N, n, m, (int64_t)pwx * 6, 0.0, buf.denseN);
    e->dense_N = buf.denseN.data();
  }
  if (d->tucker_K) {
    embed_tucker(d->tucker_K, pwx * 3, n, m, buf, buf.tkK);
    e->tucker_K = buf.tkK.data();
  } else if (d->dense_K) {
    pad_grid(d->dense_K, n, m, (int64_t)pwx * 3, 0.0, buf.denseK);
    e->dense_K = buf.denseK.data();
  }
}

}  // namespace embed
}  // namespace marie
