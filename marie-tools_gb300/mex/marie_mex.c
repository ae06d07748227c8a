/*
 * marie_mex.c -- MATLAB MEX gateway to libmarie_gb300 (the GB300 FFT-VIE
 * operator and batched GMRES).  Build inside MATLAB (R2018a+, interleaved
 * complex, Parallel Computing Toolbox for gpuArray):
 *
 *   mex -R2018a marie_mex.c -I<repo>/include -L<repo>/marie-tools_gb300/marie_gb300/lib ...
 *       -lmarie_gb300 -lcudart -lmwgpu
 *
 * Commands (first argument), mirroring the reference's call surface:
 *   h = marie_mex('create', [n1 n2 n3], PWX, res, freq, idx_solution, Mr, T [, K, precisions, max_rhs])
 *       T, K: struct arrays with fields G, U1, U2, U3 as returned by
 *       assembly_fft_circ_tucker_{pwc,pwl}.m (T(j,k) -> block j*6+k, K(j,k) -> j*3+k).
 *   Jout = marie_mex('mvp_vie', h, Jb)              % mvp_vie.m:1  (func/EP/dim bound in h)
 *   Jout = marie_mex('mvp_vie_adj', h, Jb)
 *   Jout = marie_mex('mvp_N' | 'mvp_herm_adj_N' | 'mvp_K' | 'mvp_herm_adj_K', h, Jin)
 *   [x, iter, resvec] = marie_mex('gmres', h, b, restart, tol, maxit, x0 [, mode])
 *                                                   % is_gmres_vie.m:1; b may be N_b x nrhs
 *       mode 0: FP64 (default), 1: complex64 GMRES per column + FP64 refinement,
 *       2: the same refinement with one block Krylov space for all columns
 *   marie_mex('destroy', h)
 *   hp = marie_mex('svie_pfft_create', h, N_sie, pfft_PS, pfft_Z_cc, pfft_Z_bc_N, ext_Mc_inv [, M1, M2])
 *       h: handle on the pFFT grid (MREDM.operators.pfft_N); sparse complex operands as in
 *       ie_solver_svie_pfft.m:19-26
 *   Vout = marie_mex('svie_pfft', hp, Jcb)           % mvp_svie_pfft.m:1 (operands bound in hp)
 *   marie_mex('svie_pfft_destroy', hp)
 *   Ue = marie_mex('incident_wire', h, 'E' | 'H', origin, rp, rn, r2 [, Jw])
 *       wire bases as columns rp / rn / r2 (3 x N_tri, wvie_mrgf_assembly.m:20-22), Jw N_tri x nports
 *       (default: ones); returns invG of the tested field on the body, N_b x nports
 *   I_V = marie_mex('assemble', [n1 n2 n3], PWX, res, freq, 'N' | 'K' [, 'exact' | 'standin'])
 *       assembly_N.m / assembly_K.m on the GPU, (n1, n2, n3, pwx, 6 | 3) complex; near zone 'exact'
 *       (default: the same integrals as the reference's DIRECTFN surface-surface near zone) or the
 *       'standin' cubature
 * Inputs may be host double/single complex arrays or gpuArrays; outputs follow
 * the input ('like'), as in the reference.  Errors are raised with
 * mexErrMsgIdAndTxt('marie:<status>', ...), in the style of the reference's
 * own gateways (mexAssemble_tri_coupling_matrix_N_x.cpp:13-24).
 */
#include <string.h>
#include <stdint.h>

#include "mex.h"
#include "gpu/mxGPUArray.h"
#include "marie_gb300.h"

/* cudaMemcpy without including the CUDA headers */
extern int cudaMalloc(void** p, size_t bytes);
extern int cudaFree(void* p);
extern int cudaMemcpy(void* dst, const void* src, size_t bytes, int kind);
#define H2D 1
#define D2H 2

static const char* status_id(marie_status s) {
  switch (s) {
    case MARIE_ERR_BAD_ARG: return "marie:BAD_ARG";
    case MARIE_ERR_OOM: return "marie:OOM";
    case MARIE_ERR_NONFINITE: return "marie:NONFINITE";
    case MARIE_ERR_NOT_CONVERGED: return "marie:NOT_CONVERGED";
    case MARIE_ERR_DEVICE_TIMEOUT: return "marie:DEVICE_TIMEOUT";
    case MARIE_ERR_CUDA: return "marie:CUDA";
    case MARIE_ERR_NOT_SUPPORTED: return "marie:NOT_SUPPORTED";
    default: return "marie:UNKNOWN";
  }
}

static void check(marie_status s) {
  if (s != MARIE_OK) mexErrMsgIdAndTxt(status_id(s), "%s", marie_last_error());
}

static marie_vie* get_handle(const mxArray* a) {
  if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("marie:BAD_ARG", "handle must be a uint64 scalar");
  return (marie_vie*)(uintptr_t)(*(uint64_t*)mxGetData(a));
}

static double scalar(const mxArray* a, const char* what) {
  if (!mxIsDouble(a) || mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("marie:BAD_ARG", "%s must be a double scalar", what);
  return mxGetScalar(a);
}

/* Tucker struct array -> marie_tucker_block[count]; arrays stay owned by MATLAB. */
static marie_tucker_block* tucker_blocks(const mxArray* T, int count) {
  if (!mxIsStruct(T) || (int)mxGetNumberOfElements(T) != count)
    mexErrMsgIdAndTxt("marie:BAD_ARG", "operator struct must have %d elements", count);
  marie_tucker_block* b = (marie_tucker_block*)mxCalloc(count, sizeof(marie_tucker_block));
  const int pwx_rows = (int)mxGetM(T);
  for (int id = 0; id < count; ++id) {
    /* MATLAB T(j,k) is column-major: element (j,k) at j + rows*k */
    const int ncomp = count / pwx_rows;
    const int j = id / ncomp, k = id % ncomp;
    const mwIndex e = (mwIndex)(j + pwx_rows * k);
    const mxArray* G = mxGetField(T, e, "G");
    const mxArray* U1 = mxGetField(T, e, "U1");
    const mxArray* U2 = mxGetField(T, e, "U2");
    const mxArray* U3 = mxGetField(T, e, "U3");
    if (!G || !U1 || !U2 || !U3 || !mxIsComplex(G) || !mxIsComplex(U1) || !mxIsComplex(U2) || !mxIsComplex(U3))
      mexErrMsgIdAndTxt("marie:BAD_ARG", "block %d: fields G, U1, U2, U3 must be complex double", id);
    const mwSize* d = mxGetDimensions(G);
    const mwSize nd = mxGetNumberOfDimensions(G);
    b[id].r1 = (int32_t)d[0];
    b[id].r2 = (int32_t)(nd > 1 ? d[1] : 1);
    b[id].r3 = (int32_t)(nd > 2 ? d[2] : 1);
    b[id].G = (const double*)mxGetComplexDoubles(G);
    b[id].U1 = (const double*)mxGetComplexDoubles(U1);
    b[id].U2 = (const double*)mxGetComplexDoubles(U2);
    b[id].U3 = (const double*)mxGetComplexDoubles(U3);
  }
  return b;
}

static void cmd_create(int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs) {
  if (nrhs < 8) mexErrMsgIdAndTxt("marie:BAD_ARG", "create: expected dims, PWX, res, freq, idx_solution, Mr, T");
  const double* dims = mxGetDoubles(prhs[1]);
  if (!dims || mxGetNumberOfElements(prhs[1]) != 3) mexErrMsgIdAndTxt("marie:BAD_ARG", "dims must be [n1 n2 n3]");
  marie_vie_desc d;
  memset(&d, 0, sizeof(d));
  d.n1 = (int32_t)dims[0]; d.n2 = (int32_t)dims[1]; d.n3 = (int32_t)dims[2];
  d.basis = scalar(prhs[2], "PWX") == 1 ? MARIE_PWL : MARIE_PWC;
  d.res = scalar(prhs[3], "res");
  d.freq = scalar(prhs[4], "freq");
  const mxArray* idx = prhs[5];
  const mwSize nb = mxGetNumberOfElements(idx);
  int64_t* idx0 = (int64_t*)mxCalloc(nb, sizeof(int64_t));
  const double* idxd = mxGetDoubles(idx);
  if (!idxd) mexErrMsgIdAndTxt("marie:BAD_ARG", "idx_solution must be double (1-based MATLAB indices)");
  for (mwSize i = 0; i < nb; ++i) idx0[i] = (int64_t)idxd[i] - 1;   /* MATLAB 1-based -> 0-based */
  d.n_b = (int64_t)nb;
  d.idx_solution = idx0;
  if (!mxIsComplex(prhs[6])) mexErrMsgIdAndTxt("marie:BAD_ARG", "Mr must be complex double");
  d.Mr = (const double*)mxGetComplexDoubles(prhs[6]);
  const int pwx = d.basis == MARIE_PWL ? 10 : 1;
  d.tucker_N = tucker_blocks(prhs[7], pwx * 6);
  if (nrhs > 8 && !mxIsEmpty(prhs[8])) d.tucker_K = tucker_blocks(prhs[8], pwx * 3);
  d.precisions = nrhs > 9 ? (int32_t)scalar(prhs[9], "precisions") : 3;
  d.max_rhs = nrhs > 10 ? (int32_t)scalar(prhs[10], "max_rhs") : 1;
  marie_vie* h = NULL;
  check(marie_vie_create(&h, &d));
  plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *(uint64_t*)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)h;
  (void)nlhs;
}

typedef marie_status (*apply_fn)(marie_vie*, int32_t, const void*, void*, int32_t, void*);

/* Apply an operator to a host array or a gpuArray; the output follows the input. */
static void cmd_apply(apply_fn fn, int64_t len, mxArray** plhs, const mxArray* X, marie_vie* h) {
  if (mxIsGPUArray(X)) {
    mxInitGPU();
    const mxGPUArray* x = mxGPUCreateFromMxArray(X);
    const mxClassID cls = mxGPUGetClassID(x);
    if (mxGPUGetComplexity(x) != mxCOMPLEX || (cls != mxDOUBLE_CLASS && cls != mxSINGLE_CLASS))
      mexErrMsgIdAndTxt("marie:BAD_ARG", "input must be a complex double or single gpuArray");
    const int64_t n = (int64_t)mxGPUGetNumberOfElements(x);
    if (n % len) mexErrMsgIdAndTxt("marie:BAD_ARG", "input length %lld is not a multiple of %lld", (long long)n, (long long)len);
    mxGPUArray* y = mxGPUCreateGPUArray(mxGPUGetNumberOfDimensions(x), mxGPUGetDimensions(x), cls, mxCOMPLEX,
                                        MX_GPU_DO_NOT_INITIALIZE);
    check(fn(h, cls == mxDOUBLE_CLASS ? MARIE_C128 : MARIE_C64, mxGPUGetDataReadOnly(x), mxGPUGetData(y),
             (int32_t)(n / len), NULL));
    plhs[0] = mxGPUCreateMxArrayOnGPU(y);
    mxGPUDestroyGPUArray(x);
    mxGPUDestroyGPUArray(y);
    return;
  }
  if (!mxIsComplex(X) || !mxIsDouble(X)) mexErrMsgIdAndTxt("marie:BAD_ARG", "host input must be complex double");
  const int64_t n = (int64_t)mxGetNumberOfElements(X);
  if (n % len) mexErrMsgIdAndTxt("marie:BAD_ARG", "input length is not a multiple of %lld", (long long)len);
  void *dx = NULL, *dy = NULL;
  if (cudaMalloc(&dx, (size_t)n * 16) || cudaMalloc(&dy, (size_t)n * 16)) mexErrMsgIdAndTxt("marie:OOM", "device allocation failed");
  cudaMemcpy(dx, mxGetComplexDoubles(X), (size_t)n * 16, H2D);
  marie_status s = fn(h, MARIE_C128, dx, dy, (int32_t)(n / len), NULL);
  plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(X), mxGetDimensions(X), mxDOUBLE_CLASS, mxCOMPLEX);
  if (s == MARIE_OK) cudaMemcpy(mxGetComplexDoubles(plhs[0]), dy, (size_t)n * 16, D2H);
  cudaFree(dx);
  cudaFree(dy);
  check(s);
}

static void cmd_gmres(int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs, marie_vie* h, int64_t Nb) {
  if (nrhs < 7) mexErrMsgIdAndTxt("marie:BAD_ARG", "gmres: expected h, b, restart, tol, maxit, x0");
  const mxArray* B = prhs[2];
  if (mxIsGPUArray(B) || !mxIsComplex(B)) mexErrMsgIdAndTxt("marie:BAD_ARG", "b must be a host complex double array");
  const int64_t n = (int64_t)mxGetNumberOfElements(B);
  const int32_t k = (int32_t)(n / Nb);
  marie_gmres_opts o;
  memset(&o, 0, sizeof(o));
  o.restart = (int32_t)scalar(prhs[3], "restart");
  o.tol = scalar(prhs[4], "tol");
  o.maxit = (int32_t)scalar(prhs[5], "maxit");
  o.mode = nrhs > 7 ? (int32_t)scalar(prhs[7], "mode") : MARIE_SOLVE_FP64;
  o.inner_tol = 0.0;      /* library defaults */
  o.max_refine = 0;
  o.inner_safety = 0.0;
  const mxArray* X0 = prhs[6];
  /* the solution array doubles as x0: the host-buffer solve reads it when
     x0_present and overwrites it with the solution */
  plhs[0] = mxCreateNumericArray(mxGetNumberOfDimensions(B), mxGetDimensions(B), mxDOUBLE_CLASS, mxCOMPLEX);
  if (!mxIsEmpty(X0) && mxIsComplex(X0) && (int64_t)mxGetNumberOfElements(X0) == n) {
    memcpy(mxGetComplexDoubles(plhs[0]), mxGetComplexDoubles(X0), (size_t)n * 16);
    o.x0_present = 1;
  }
  const int cap = o.restart * (o.maxit > 0 ? o.maxit : 1) + 1;
  int32_t* outer = (int32_t*)mxCalloc(k, sizeof(int32_t));
  int32_t* last = (int32_t*)mxCalloc(k, sizeof(int32_t));
  int32_t* rlen = (int32_t*)mxCalloc(k, sizeof(int32_t));
  double* rv = (double*)mxCalloc((size_t)k * cap, sizeof(double));
  marie_gmres_report rep;
  memset(&rep, 0, sizeof(rep));
  rep.outer = outer;
  rep.last_inner = last;
  rep.resvec = rv;
  rep.resvec_cap = cap;
  rep.resvec_len = rlen;
  /* host arrays straight into the chunked host-buffer solve */
  marie_status s = marie_gmres_vie_host(h, mxGetComplexDoubles(B), mxGetComplexDoubles(plhs[0]), k, &o, &rep, NULL);
  if (s != MARIE_OK && s != MARIE_ERR_NOT_CONVERGED) check(s);
  if (nlhs > 1) {
    plhs[1] = mxCreateDoubleMatrix(k, 2, mxREAL);   /* iter = [p outit] per rhs */
    double* it = mxGetDoubles(plhs[1]);
    for (int r = 0; r < k; ++r) { it[r] = last[r]; it[r + k] = outer[r]; }
  }
  if (nlhs > 2) {
    int mx = 0;
    for (int r = 0; r < k; ++r) mx = rlen[r] > mx ? rlen[r] : mx;
    plhs[2] = mxCreateDoubleMatrix(mx, k, mxREAL);
    double* o2 = mxGetDoubles(plhs[2]);
    for (int r = 0; r < k; ++r)
      for (int i = 0; i < rlen[r]; ++i) o2[i + (size_t)mx * r] = rv[(size_t)r * cap + i];
  }
}

/* I_V = marie_mex('assemble', [n1 n2 n3], PWX, res, freq, kernel [, near]) */
static void cmd_assemble(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  (void)nlhs;
  if (nrhs < 6) mexErrMsgIdAndTxt("marie:BAD_ARG", "assemble needs [n1 n2 n3], PWX, res, freq, 'N'|'K'");
  if (!mxIsDouble(prhs[1]) || mxGetNumberOfElements(prhs[1]) != 3)
    mexErrMsgIdAndTxt("marie:BAD_ARG", "grid size must be a 1x3 double");
  const double* nd = mxGetDoubles(prhs[1]);
  const int32_t n1 = (int32_t)nd[0], n2 = (int32_t)nd[1], n3 = (int32_t)nd[2];
  const int pwl = scalar(prhs[2], "PWX") == 1.0;
  const double res = scalar(prhs[3], "res"), freq = scalar(prhs[4], "freq");
  char kern[8] = {0}, near[16] = {0};
  if (!mxIsChar(prhs[5]) || mxGetString(prhs[5], kern, sizeof(kern)) || (strcmp(kern, "N") && strcmp(kern, "K")))
    mexErrMsgIdAndTxt("marie:BAD_ARG", "kernel must be 'N' or 'K'");
  int32_t flags = MARIE_GREEN_NEAR_EXACT;
  if (nrhs > 6) {
    if (!mxIsChar(prhs[6]) || mxGetString(prhs[6], near, sizeof(near)) ||
        (strcmp(near, "exact") && strcmp(near, "standin")))
      mexErrMsgIdAndTxt("marie:BAD_ARG", "near zone must be 'exact' or 'standin'");
    if (!strcmp(near, "standin")) flags = 0;
  }
  if (n1 < 1 || n2 < 1 || n3 < 1) mexErrMsgIdAndTxt("marie:BAD_ARG", "grid edges must be positive");
  const mwSize dims[5] = {(mwSize)n1, (mwSize)n2, (mwSize)n3, (mwSize)(pwl ? 10 : 1), (mwSize)(kern[0] == 'N' ? 6 : 3)};
  plhs[0] = mxCreateNumericArray(5, dims, mxDOUBLE_CLASS, mxCOMPLEX);
  check(marie_assemble_green_ex(n1, n2, n3, res, freq, pwl ? MARIE_PWL : MARIE_PWC, kern[0] == 'N' ? 0 : 1, flags,
                                (double*)mxGetComplexDoubles(plhs[0])));
}

/* MATLAB sparse (compressed columns, 1 column pointer per column) -> CSR
 * with 0-based indices; arrays allocated with mxCalloc. */
static marie_csr sparse_to_csr(const mxArray* A, const char* what) {
  if (!mxIsSparse(A) || !mxIsDouble(A)) mexErrMsgIdAndTxt("marie:BAD_ARG", "%s must be a sparse double matrix", what);
  const mwSize m = mxGetM(A), n = mxGetN(A);
  const mwIndex* jc = mxGetJc(A);
  const mwIndex* ir = mxGetIr(A);
  const mwIndex nnz = jc[n];
  const int cplx = mxIsComplex(A);
  const double* re = cplx ? NULL : mxGetDoubles(A);
  const mxComplexDouble* cz = cplx ? mxGetComplexDoubles(A) : NULL;
  int64_t* rp = (int64_t*)mxCalloc(m + 1, sizeof(int64_t));
  int64_t* ci = (int64_t*)mxCalloc(nnz > 0 ? nnz : 1, sizeof(int64_t));
  double* v = (double*)mxCalloc(2 * (nnz > 0 ? nnz : 1), sizeof(double));
  for (mwIndex k = 0; k < nnz; ++k) rp[ir[k] + 1]++;
  for (mwSize r = 0; r < m; ++r) rp[r + 1] += rp[r];
  int64_t* next = (int64_t*)mxCalloc(m > 0 ? m : 1, sizeof(int64_t));
  for (mwSize r = 0; r < m; ++r) next[r] = rp[r];
  for (mwSize c = 0; c < n; ++c)
    for (mwIndex k = jc[c]; k < jc[c + 1]; ++k) {
      const int64_t d = next[ir[k]]++;
      ci[d] = (int64_t)c;
      v[2 * d] = cplx ? cz[k].real : re[k];
      v[2 * d + 1] = cplx ? cz[k].imag : 0.0;
    }
  marie_csr out;
  out.rows = (int64_t)m;
  out.cols = (int64_t)n;
  out.nnz = (int64_t)nnz;
  out.row_ptr = rp;
  out.col_idx = ci;
  out.val = v;
  return out;
}

static void cmd_svie_pfft_create(mxArray** plhs, int nrhs, const mxArray** prhs) {
  if (nrhs < 7) mexErrMsgIdAndTxt("marie:BAD_ARG", "svie_pfft_create: expected h, N_sie, PS, Z_cc, Z_bc_N, ext_Mc_inv");
  marie_svie_pfft_desc d;
  memset(&d, 0, sizeof(d));
  d.grid_op = get_handle(prhs[1]);
  d.n_sie = (int64_t)scalar(prhs[2], "N_sie");
  d.PS = sparse_to_csr(prhs[3], "pfft_PS");
  d.n_b = d.PS.cols - d.n_sie;
  d.Z_cc = sparse_to_csr(prhs[4], "pfft_Z_cc");
  d.Z_bc_N = sparse_to_csr(prhs[5], "pfft_Z_bc_N");
  if (!mxIsComplex(prhs[6]) || !mxIsDouble(prhs[6])) mexErrMsgIdAndTxt("marie:BAD_ARG", "ext_Mc_inv must be complex double");
  d.ext_Mc_inv = (const double*)mxGetComplexDoubles(prhs[6]);
  if (nrhs > 7 && !mxIsEmpty(prhs[7])) d.M1 = mxGetDoubles(prhs[7]);
  if (nrhs > 8 && !mxIsEmpty(prhs[8])) d.M2 = mxGetDoubles(prhs[8]);
  marie_svie_pfft* hp = NULL;
  check(marie_svie_pfft_create(&hp, &d));
  plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *(uint64_t*)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)hp;
}

static marie_status svie_pfft_apply_as_vie(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs,
                                           void* stream) {
  return marie_svie_pfft_apply((marie_svie_pfft*)(void*)h, prec, x, y, nrhs, stream);
}

/* Ue = marie_mex('incident_wire', h, 'E'|'H', origin, rp, rn, r2 [, Jw]) */
static void cmd_incident_wire(mxArray** plhs, int nrhs, const mxArray** prhs, marie_vie* h) {
  if (nrhs < 7) mexErrMsgIdAndTxt("marie:BAD_ARG", "incident_wire: expected h, 'E'|'H', origin, rp, rn, r2");
  char kind[4] = {0};
  if (!mxIsChar(prhs[2]) || mxGetString(prhs[2], kind, sizeof(kind)) || (strcmp(kind, "E") && strcmp(kind, "H")))
    mexErrMsgIdAndTxt("marie:BAD_ARG", "field must be 'E' or 'H'");
  const double* org = mxGetDoubles(prhs[3]);
  if (!org || mxGetNumberOfElements(prhs[3]) != 3) mexErrMsgIdAndTxt("marie:BAD_ARG", "origin must be 3 doubles");
  const int32_t ntri = (int32_t)mxGetN(prhs[4]);
  for (int i = 4; i < 7; ++i)
    if (!mxIsDouble(prhs[i]) || mxGetM(prhs[i]) != 3 || (int32_t)mxGetN(prhs[i]) != ntri)
      mexErrMsgIdAndTxt("marie:BAD_ARG", "rp, rn, r2 must be 3 x N_tri doubles");
  const double* cf = NULL;
  int32_t nports = 1;
  if (nrhs > 7 && !mxIsEmpty(prhs[7])) {
    const mxArray* J = prhs[7];
    if (!mxIsComplex(J) || (int32_t)mxGetM(J) != ntri) mexErrMsgIdAndTxt("marie:BAD_ARG", "Jw must be complex N_tri x nports");
    nports = (int32_t)mxGetN(J);
    cf = (const double*)mxGetComplexDoubles(J);     /* column p = port p: nports x N_tri row-major */
  }
  int64_t info[6];
  check(marie_vie_info(h, info));
  const int64_t Nb = info[5];
  void* d = NULL;
  if (cudaMalloc(&d, (size_t)Nb * nports * 16)) mexErrMsgIdAndTxt("marie:OOM", "device allocation failed");
  marie_status st = marie_incident_wire(h, kind[0] == 'E' ? 0 : 1, org, mxGetDoubles(prhs[4]), mxGetDoubles(prhs[5]),
                                        mxGetDoubles(prhs[6]), ntri, cf, nports, 4, 2, d, NULL);
  plhs[0] = mxCreateNumericMatrix((mwSize)Nb, (mwSize)nports, mxDOUBLE_CLASS, mxCOMPLEX);
  if (st == MARIE_OK) cudaMemcpy(mxGetComplexDoubles(plhs[0]), d, (size_t)Nb * nports * 16, D2H);
  cudaFree(d);
  check(st);
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs < 1 || !mxIsChar(prhs[0])) mexErrMsgIdAndTxt("marie:BAD_ARG", "first argument must be a command string");
  char cmd[32];
  mxGetString(prhs[0], cmd, sizeof(cmd));
  if (!strcmp(cmd, "create")) { cmd_create(nlhs, plhs, nrhs, prhs); return; }
  if (!strcmp(cmd, "assemble")) { cmd_assemble(nlhs, plhs, nrhs, prhs); return; }
  if (nrhs < 2) mexErrMsgIdAndTxt("marie:BAD_ARG", "missing handle");
  marie_vie* h = get_handle(prhs[1]);
  if (!strcmp(cmd, "destroy")) { check(marie_vie_destroy(h)); return; }
  if (!strcmp(cmd, "svie_pfft_create")) { cmd_svie_pfft_create(plhs, nrhs, prhs); return; }
  if (!strcmp(cmd, "svie_pfft_destroy")) { check(marie_svie_pfft_destroy((marie_svie_pfft*)(void*)h)); return; }
  if (!strcmp(cmd, "incident_wire")) { cmd_incident_wire(plhs, nrhs, prhs, h); return; }
  /* lengths: body vector N_b is taken from the input length per rhs via the handle's apply checks */
  if (nrhs < 3) mexErrMsgIdAndTxt("marie:BAD_ARG", "missing input array");
  const mwSize* d = mxGetDimensions(prhs[2]);
  const int64_t rows = (int64_t)d[0];
  if (!strcmp(cmd, "mvp_vie")) { cmd_apply(marie_vie_apply, rows, plhs, prhs[2], h); return; }
  if (!strcmp(cmd, "mvp_vie_adj")) { cmd_apply(marie_vie_apply_adjoint, rows, plhs, prhs[2], h); return; }
  if (!strcmp(cmd, "gmres")) { cmd_gmres(nlhs, plhs, nrhs, prhs, h, rows); return; }
  if (!strcmp(cmd, "svie_pfft")) { cmd_apply(svie_pfft_apply_as_vie, rows, plhs, prhs[2], h); return; }
  /* grid operators: Jin is n1 x n2 x n3 x C */
  const int64_t grid = (int64_t)mxGetNumberOfElements(prhs[2]);
  if (!strcmp(cmd, "mvp_N")) { cmd_apply(marie_vie_apply_N, grid, plhs, prhs[2], h); return; }
  if (!strcmp(cmd, "mvp_herm_adj_N")) { cmd_apply(marie_vie_apply_N_adj, grid, plhs, prhs[2], h); return; }
  if (!strcmp(cmd, "mvp_K")) { cmd_apply(marie_vie_apply_K, grid, plhs, prhs[2], h); return; }
  if (!strcmp(cmd, "mvp_herm_adj_K")) { cmd_apply(marie_vie_apply_K_adj, grid, plhs, prhs[2], h); return; }
  mexErrMsgIdAndTxt("marie:BAD_ARG", "unknown command '%s'", cmd);
}
