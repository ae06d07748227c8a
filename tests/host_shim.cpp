// C entry points over the host-only helpers of the library (grid embedding,
// marie-tools_gb300/csrc/embed.h; the Green's-tensor self point term,
// marie-tools_gb300/csrc/green_host.h), compiled with g++ by the CPU tests
// (tests/test_embed_host.py, tests/test_green_host.py) so that the helpers
// are checked against numpy and the oracle.
#include "../marie-tools_gb300/csrc/embed.h"
#include "../marie-tools_gb300/csrc/green_host.h"

extern "C" {
int shim_embed_dims(const int* n, int force, int* m) { return marie::embed::embed_dims(n, force != 0, m) ? 1 : 0; }
void shim_embed_factor(const double* U, int r, int n, int m, double* out) {
  std::vector<double> o;
  marie::embed::embed_factor(U, r, n, m, o);
  std::memcpy(out, o.data(), o.size() * sizeof(double));
}
void shim_pad_grid(const double* src, const int* n, const int* m, long long nblk, double fill, double* out) {
  std::vector<double> o;
  marie::embed::pad_grid(src, n, m, nblk, fill, o);
  std::memcpy(out, o.data(), o.size() * sizeof(double));
}
void shim_add_self_point_term(double* out, long long nD, int pwx, double res) {
  marie::green_host::add_self_point_term(out, nD, pwx, res);
}
void shim_near_zone_exact(double* iv, int n1, int n2, int n3, double res, double k0, int pwx, int isN, int order) {
  marie::green_host::near_zone_exact(iv, n1, n2, n3, res, k0, pwx, isN != 0, order);
}
void shim_gauss01(int n, double* x, double* w) {
  std::vector<double> xv, wv;
  marie::green_host::gauss01(n, xv, wv);
  for (int i = 0; i < n; ++i) { x[i] = xv[i]; w[i] = wv[i]; }
}
long long shim_remap(long long lin, const int* n, const int* m) { return marie::embed::remap_voxel(lin, n, m); }
}
