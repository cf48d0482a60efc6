// NSYSLV ISOLV=-5 (Jacobi-preconditioned BiCGSTAB) for callers that cannot
// allocate device memory.
//
// Some host programs may not call cudaMalloc once they are running: a
// Fortran driver whose device memory is owned by a host framework with its
// own pool, or code that must not allocate between steps.  This entry point
// runs the same solve as cathy_gb300_nsyslv(ISOLV=-5) on matrix, right-hand
// side and solution buffers that the caller already holds in device memory,
// and keeps every piece of solver workspace in one fixed, file-scope device
// array.  It calls no cudaMalloc, cudaFree or allocating library routine.
//
// The array is loaded with the library on every GPU the process uses and
// stays resident until the process exits; it limits the system size to
// CATHY_GB300_NOALLOC_MAXN rows.  All calls share it and it keeps the last
// call's contents, so each call clears what must start at zero, and calls
// that overlap on the GPU (two streams, or two host threads) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/cathy_gb300.h"

namespace {

constexpr int kMaxN = CATHY_GB300_NOALLOC_MAXN;
constexpr int kNumVec = 9;      // r, rt, p, v, s, t, pjm, vjm, dinv
constexpr int kNumScal = 64;    // reduction slots and iteration state
constexpr int kMaskDoubles = kMaxN / 8;  // one byte per row
constexpr long kScratchDoubles = (long)kNumVec * kMaxN + kMaskDoubles + kNumScal;
constexpr int kThreads = 256;
constexpr int kLanes = 16;      // lanes per matrix row in the row products

// The workspace.  Host code must not take this name as a device address:
// the address comes from cudaGetSymbolAddress (scratch_address below).
static __device__ __align__(256) double g_scratch[kScratchDoubles];

// scalar slots (after the vectors and the mask)
enum {
  S_XL = 0, S_ROJ, S_SIG, S_AA, S_BB, S_RR, S_ROJM1, S_ALFJM1, S_ETAJ, S_ERR,
  S_TRR, S_TBB, S_NITER, S_ACTIVE, S_BN
};

struct Work {
  double *r, *rt, *p, *v, *s, *t, *pjm, *vjm, *dinv;
  unsigned char* dm;
  double* sc;
};

Work carve(double* base) {
  Work w;
  double* q = base;
  w.r = q; q += kMaxN;
  w.rt = q; q += kMaxN;
  w.p = q; q += kMaxN;
  w.v = q; q += kMaxN;
  w.s = q; q += kMaxN;
  w.t = q; q += kMaxN;
  w.pjm = q; q += kMaxN;
  w.vjm = q; q += kMaxN;
  w.dinv = q; q += kMaxN;
  w.dm = reinterpret_cast<unsigned char*>(q); q += kMaskDoubles;
  w.sc = q;
  return w;
}

// ---- per-device set-up: the device address of g_scratch -------------------
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Called with the caller's device current.  The first call on a device asks
// the runtime for the symbol's device address; later calls reuse it.
cudaError_t scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<double*>(ptr);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

// ---- kernels (one system, rows [0, n)) -------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// block sum of NV values, one atomic per value into acc[0..NV)
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* acc) {
  __shared__ double sh[NV][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < NV; ++i) {
    const double s = warp_sum(v[i]);
    if (lane == 0) sh[i][w] = s;
  }
  __syncthreads();
  if (w == 0) {
    for (int i = 0; i < NV; ++i) {
      double s = lane < (kThreads / 32) ? sh[i][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0 && s != 0.0) atomicAdd(acc + i, s);
    }
  }
}

__global__ void k_clear(int n, Work w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kNumScal) {
    // rojm1 = alfjm1 = etaj = 1 as GCSTAD starts; iteration count 1; active
    const bool one = i == S_ROJM1 || i == S_ALFJM1 || i == S_ETAJ || i == S_NITER ||
                     i == S_ACTIVE;
    w.sc[i] = one ? 1.0 : 0.0;
  }
  if (i < n) {
    w.dm[i] = 0;
    w.pjm[i] = 0.0;
    w.vjm[i] = 0.0;
  }
}

// Dirichlet mask from the reference's 1-based NODDIR list
__global__ void k_mark(int numdir, const int32_t* noddir, int n, Work w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < numdir) {
    const int i = noddir[k] - 1;
    if (i >= 0 && i < n) w.dm[i] = 1;
  }
}

// dinv = 1/a_ii (1 at Dirichlet rows); x0 = dinv*b; xl = |b_masked|^2 (the
// error norm's denominator) and, in its own slot, the sum of TNOTI^2 over
// every row, Dirichlet rows included (NSYSLV's zero right-hand-side test)
__global__ void k_setup(int n, const int32_t* topol, const int32_t* ja, const double* a,
                        const double* tnoti, double* x, Work w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0}, u[1] = {0.0};
  if (i < n) {
    double d = 1.0;
    if (!w.dm[i]) {
      for (int q = topol[i] - 1; q < topol[i + 1] - 1; ++q)
        if (ja[q] - 1 == i) d = a[q];
      d = 1.0 / d;
    }
    w.dinv[i] = d;
    const double b = w.dm[i] ? 0.0 : tnoti[i];
    x[i] = d * b;
    v[0] = b * b;
    u[0] = tnoti[i] * tnoti[i];
  }
  block_sum<1>(v, w.sc + S_XL);
  block_sum<1>(u, w.sc + S_BN);
}

// out = dinv * (A in) with Dirichlet rows as identity (16 lanes per row);
// mode 1: out = dinv * (b - A in) (initial residual)
__global__ void k_jspmv(int n, const int32_t* topol, const int32_t* ja, const double* a,
                        const double* in, double* out, const double* tnoti, int mode, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / kLanes;
  const int lane = threadIdx.x % kLanes;
  double s = 0.0;
  if (row < n) {
    for (int q = topol[row] - 1 + lane; q < topol[row + 1] - 1; q += kLanes)
      s += a[q] * in[ja[q] - 1];
  }
  for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (row < n && lane == 0) {
    double y = w.dm[row] ? in[row] : s;
    if (mode == 1) y = (w.dm[row] ? 0.0 : tnoti[row]) - y;
    out[row] = w.dinv[row] * y;
  }
}

__global__ void k_dot(int n, const double* a, const double* b, int slot, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (i < n) v[0] = a[i] * b[i];
  block_sum<1>(v, w.sc + slot);
}

__global__ void k_copy(int n, const double* a, double* b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// p = r + beta (pjm - etaj vjm)
__global__ void k_pdir(int n, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* S = w.sc;
  const double beta = (S[S_ROJ] / S[S_ROJM1]) * (S[S_ALFJM1] / S[S_ETAJ]);
  w.p[i] = w.r[i] + beta * (w.pjm[i] - S[S_ETAJ] * w.vjm[i]);
}

// s = r - alf v
__global__ void k_sdir(int n, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  w.s[i] = w.r[i] - (w.sc[S_ROJ] / w.sc[S_SIG]) * w.v[i];
}

// aa = s.t, bb = t.t
__global__ void k_st(int n, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    v[0] = w.s[i] * w.t[i];
    v[1] = w.t[i] * w.t[i];
  }
  block_sum<2>(v, w.sc + S_AA);
}

// x += alf p + eta s; r = s - eta t (zero at Dirichlet rows); rr = |r|^2;
// then pjm = p, vjm = v for the next iteration
__global__ void k_xr(int n, double* x, Work w) {
  if (w.sc[S_ACTIVE] == 0.0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (i < n) {
    const double alf = w.sc[S_ROJ] / w.sc[S_SIG];
    const double eta = w.sc[S_AA] / w.sc[S_BB];
    x[i] = x[i] + alf * w.p[i] + eta * w.s[i];
    const double ri = w.dm[i] ? 0.0 : w.s[i] - eta * w.t[i];
    w.r[i] = ri;
    v[0] = ri * ri;
    w.pjm[i] = w.p[i];
    w.vjm[i] = w.v[i];
  }
  block_sum<1>(v, w.sc + S_RR);
}

// GCSTAD's convergence test and the scalar recurrences of the next
// iteration; clears the per-iteration reduction slots.
__global__ void k_decide(int itmax, double tol, Work w) {
  double* S = w.sc;
  if (S[S_ACTIVE] == 0.0) return;
  const double xl = S[S_XL];
  const double err = xl > 0.0 ? sqrt(S[S_RR] / xl) : 0.0;
  S[S_ERR] = err;
  const int niter = (int)S[S_NITER];
  if (niter <= itmax && err > tol) {
    S[S_ROJM1] = S[S_ROJ];
    S[S_ALFJM1] = S[S_ROJ] / S[S_SIG];
    S[S_ETAJ] = S[S_AA] / S[S_BB];
    S[S_NITER] = niter + 1;
  } else {
    S[S_ACTIVE] = 0.0;
  }
  S[S_ROJ] = S[S_SIG] = S[S_AA] = S[S_BB] = S[S_RR] = 0.0;
}

// true residual |b - A x| / |b| over non-Dirichlet rows and columns
__global__ void k_true_resid(int n, const int32_t* topol, const int32_t* ja, const double* a,
                             const double* tnoti, const double* x, Work w) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / kLanes;
  const int lane = threadIdx.x % kLanes;
  double s = 0.0;
  const bool ok = row < n && !w.dm[row];
  if (ok) {
    for (int q = topol[row] - 1 + lane; q < topol[row + 1] - 1; q += kLanes) {
      const int j = ja[q] - 1;
      if (!w.dm[j]) s += a[q] * x[j];
    }
  }
  for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  double v[2] = {0.0, 0.0};
  if (ok && lane == 0) {
    const double ri = tnoti[row] - s;
    v[0] = ri * ri;
    v[1] = tnoti[row] * tnoti[row];
  }
  block_sum<2>(v, w.sc + S_TRR);
}

inline int blocks(long work, int per) { return (int)((work + per - 1) / per); }

int fail(cudaError_t e, const char* where) {
  fprintf(stderr, "cathy_gb300_nsyslv_noalloc: %s: %s\n", where, cudaGetErrorString(e));
  return CATHY_GB300_ENODEV;
}

}  // namespace

extern "C" int32_t cathy_gb300_nsyslv_noalloc(
    const int32_t* n_, const int32_t* numdir_, const int32_t* noddir_d,
    const int32_t* itmxcg_, int32_t* niter, const int32_t* ja_d, const int32_t* topol_d,
    const double* tolcg_, const double* coef1_d, double* pnew_d, const double* tnoti_d,
    double* err, double* res, void* stream) {
  if (!n_ || !numdir_ || !itmxcg_ || !niter || !ja_d || !topol_d || !tolcg_ || !coef1_d ||
      !pnew_d || !tnoti_d || *n_ <= 0 || *numdir_ < 0 || (*numdir_ > 0 && !noddir_d))
    return CATHY_GB300_EINVAL;
  const int n = *n_, numdir = *numdir_, itmax = *itmxcg_;
  const double tol = *tolcg_;
  if (n > kMaxN) {
    fprintf(stderr,
            "cathy_gb300_nsyslv_noalloc: n = %d exceeds the fixed workspace limit "
            "CATHY_GB300_NOALLOC_MAXN = %d rows; use cathy_gb300_nsyslv\n", n, kMaxN);
    return CATHY_GB300_EINVAL;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CATHY_GB300_ENODEV;
  double* base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) return fail(e, "cudaGetSymbolAddress");
  const Work w = carve(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int gn = blocks(n, kThreads), gr = blocks((long)n * kLanes, kThreads);

  k_clear<<<blocks(n > kNumScal ? n : kNumScal, kThreads), kThreads, 0, st>>>(n, w);
  if (numdir > 0) k_mark<<<blocks(numdir, kThreads), kThreads, 0, st>>>(numdir, noddir_d, n, w);
  k_setup<<<gn, kThreads, 0, st>>>(n, topol_d, ja_d, coef1_d, tnoti_d, pnew_d, w);
  // a launch that failed without a sticky error (no kernel image for the
  // device, say) would otherwise leave the copy below reading a slot that
  // nothing wrote
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "set-up launch");
  double bn = 0.0;
  if ((e = cudaMemcpyAsync(&bn, w.sc + S_BN, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(e, "set-up");
  if (bn == 0.0) {  // NSYSLV returns PNEW = 0 when every TNOTI is zero
    if ((e = cudaMemsetAsync(pnew_d, 0, sizeof(double) * n, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail(e, "zero solution");
    *niter = 0;
    if (err) *err = 0.0;
    if (res) *res = 0.0;
    return CATHY_GB300_OK;
  }
  // r0 = D^-1 (b - A x0), rt = r0 (GCSTAD with the diagonal scaling of PRDY)
  k_jspmv<<<gr, kThreads, 0, st>>>(n, topol_d, ja_d, coef1_d, pnew_d, w.r, tnoti_d, 1, w);
  k_copy<<<gn, kThreads, 0, st>>>(n, w.r, w.rt);
  for (int it = 0; it < itmax + 3; ++it) {
    k_dot<<<gn, kThreads, 0, st>>>(n, w.rt, w.r, S_ROJ, w);
    k_pdir<<<gn, kThreads, 0, st>>>(n, w);
    k_jspmv<<<gr, kThreads, 0, st>>>(n, topol_d, ja_d, coef1_d, w.p, w.v, nullptr, 0, w);
    k_dot<<<gn, kThreads, 0, st>>>(n, w.rt, w.v, S_SIG, w);
    k_sdir<<<gn, kThreads, 0, st>>>(n, w);
    k_jspmv<<<gr, kThreads, 0, st>>>(n, topol_d, ja_d, coef1_d, w.s, w.t, nullptr, 0, w);
    k_st<<<gn, kThreads, 0, st>>>(n, w);
    k_xr<<<gn, kThreads, 0, st>>>(n, pnew_d, w);
    k_decide<<<1, 1, 0, st>>>(itmax, tol, w);
    double active = 0.0;
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "launch");
    if ((e = cudaMemcpyAsync(&active, w.sc + S_ACTIVE, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail(e, "iteration");
    if (active == 0.0) break;
  }
  k_true_resid<<<gr, kThreads, 0, st>>>(n, topol_d, ja_d, coef1_d, tnoti_d, pnew_d, w);
  double sc[kNumScal];
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "launch");
  if ((e = cudaMemcpyAsync(sc, w.sc, sizeof(sc), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(e, "results");
  *niter = (int32_t)sc[S_NITER];
  if (err) *err = sc[S_ERR];
  if (res) *res = sc[S_TBB] > 1.7e-100 ? std::sqrt(sc[S_TRR] / sc[S_TBB]) : std::sqrt(sc[S_TRR] / n);
  return CATHY_GB300_OK;
}
