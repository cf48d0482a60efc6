// Learned column-line preconditioner: feature, network (forward/backward),
// loss and Adam kernels.  See learned.h for the model.
//
// Row kernels give one warp one matrix row: the row's slots (at most 16,
// the longest row of a P1 tetrahedral extruded mesh has 15) form the 16 rows
// of an m16n8k16 BF16 tensor-core tile, so a node's messages are reduced
// inside the warp with shuffles.  Activations move between layers in
// registers (the accumulator fragment of one layer is the A fragment of the
// next).  Weight gradients are sums over slots: four warps stage their tiles
// in shared memory and each warp accumulates a 16-channel slice of the
// gradient on the tensor cores across the whole grid-stride loop.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "engine.h"
#include "learned.h"

namespace cathy {

namespace {

constexpr int kWarps = 4;
constexpr int kBlock = 32 * kWarps;

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(uint16_t lo, uint16_t hi) {
  return (uint32_t)lo | ((uint32_t)hi << 16);
}
__device__ __forceinline__ float bfr(float x) {
  return __bfloat162float(__float2bfloat16_rn(x));
}
__device__ __forceinline__ uint16_t bfbits(float x) {
  __nv_bfloat16 b = __float2bfloat16_rn(x);
  return *reinterpret_cast<uint16_t*>(&b);
}

// D += A B, m16n8k16, BF16 inputs, FP32 accumulation
__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Weights staged in shared memory by every row kernel.
struct SmemW {
  uint16_t W1[kLpHid * kLpNF];
  uint16_t W2[kLpHid * kLpHid];
  uint16_t W2t[kLpHid * kLpHid];
  float b1[kLpHid], b2[kLpHid], w3[kLpHid];
  float b3;
};

__device__ void load_weights(SmemW& s, const uint16_t* wbf, const float* P) {
  const int nW1 = kLpHid * kLpNF, nW2 = kLpHid * kLpHid;
  for (int q = threadIdx.x; q < nW1; q += blockDim.x) s.W1[q] = wbf[q];
  for (int q = threadIdx.x; q < nW2; q += blockDim.x) {
    s.W2[q] = wbf[nW1 + q];
    s.W2t[q] = wbf[nW1 + nW2 + q];
  }
  for (int q = threadIdx.x; q < kLpHid; q += blockDim.x) {
    s.b1[q] = P[kLpOffB1 + q];
    s.b2[q] = P[kLpOffB2 + q];
    s.w3[q] = P[kLpOffW3 + q];
  }
  if (threadIdx.x == 0) s.b3 = P[kLpOffB3];
  __syncthreads();
}

// Per-row context of the warp.
struct RowCtx {
  int i, s0, len, sd, m, nn;
  bool dmi, ok;
};

__device__ __forceinline__ RowCtx row_ctx(const LpGraph& g, int i) {
  RowCtx r;
  r.i = i;
  r.ok = false;
  r.s0 = r.len = r.sd = r.m = r.nn = 0;
  r.dmi = true;
  if (i < g.n) {
    r.m = g.mem[i];
    if (g.active[r.m]) {
      r.ok = true;
      r.s0 = g.rowptr[i];
      r.len = g.rowptr[i + 1] - r.s0;
      r.sd = g.diag[i];
      r.nn = g.nnod[r.m];
      r.dmi = g.dmask[i] != 0;
    }
  }
  return r;
}

__device__ __forceinline__ bool slot_valid(const RowCtx& r, int row) {
  return r.ok && row < r.len && r.s0 + row != r.sd;
}

// node features: (rowsum/a_ii, log10 Ks, scaled log10 cap, sqrt|a_ii|)
__global__ void k_lp_nodes(LpGraph g, float4* node4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n || !g.active[g.mem[i]]) return;
  const int s0 = g.rowptr[i], s1 = g.rowptr[i + 1];
  const float d = g.vals[g.diag[i]];
  float rs = 0.0f;
  for (int s = s0; s < s1; ++s)
    if (!g.dmask[g.cols[s]]) rs += g.vals[s];
  const bool dm = g.dmask[i] != 0;
  float4 v;
  v.x = dm ? 1.0f : rs / d;
  v.y = log10f(g.ks[i]);
  v.z = log10f(g.pnodi[i] * g.et2[i] + 1e-7f) * (1.0f / 3.0f) + 1.0f;
  v.w = sqrtf(fabsf(d));
  node4[i] = v;
}

// The two features (2t, 2t+1) of tile row `row` (zero for invalid rows).
__device__ __forceinline__ float2 feat_pair(const LpGraph& g, const float4* node4,
                                            const RowCtx& r, int row, int t, float& aij,
                                            int& j) {
  aij = 0.0f;
  j = -1;
  if (!slot_valid(r, row)) return make_float2(0.0f, 0.0f);
  const int s = r.s0 + row;
  j = g.cols[s];
  aij = g.vals[s];
  const float4 ni = node4[r.i], nj = node4[j];
  switch (t) {
    case 0: {
      const bool dmj = g.dmask[j] != 0;
      const float c = (r.dmi || dmj) ? 0.0f : aij / (ni.w * nj.w);
      return make_float2(c, ni.x);
    }
    case 1:
      return make_float2(nj.x, (ni.y + 5.0f) * 0.5f);
    case 2:
      return make_float2(ni.z, log10f(g.dt[r.m]) * 0.5f - 1.0f);
    default: {
      const int dij = j - r.i;
      const float vert = (dij == r.nn || dij == -r.nn) ? 1.0f : 0.0f;
      return make_float2(vert, (nj.y - ni.y) * 0.5f);
    }
  }
}

// Layer 1 for the warp's tile: z1 (pre-activation) and h1 = bf16(relu(z1)).
// fa: features (2t, 2t+1) of rows g and g+8.
__device__ __forceinline__ void layer1(const SmemW& W, float2 fg, float2 fg8, int g, int t,
                                       float (&z1)[8][4], float (&h1)[8][4]) {
  const uint32_t a0 = pack2(fg.x, fg.y), a1 = pack2(fg8.x, fg8.y);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int nrow = 8 * c + g;
    const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&W.W1[nrow * kLpNF + 2 * t]);
    const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&W.W1[nrow * kLpNF + 2 * t + 8]);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(acc, a0, a1, 0u, 0u, b0, b1);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float z = acc[q] + W.b1[8 * c + 2 * t + (q & 1)];
      z1[c][q] = z;
      h1[c][q] = bfr(fmaxf(z, 0.0f));
    }
  }
}

// Layer 2 from U (given as fp32 values already rounded to bf16): z2.
__device__ __forceinline__ void layer2(const SmemW& W, const float (&u)[8][4], int g, int t,
                                       float (&z2)[8][4]) {
  uint32_t a[4][4];
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    a[kk][0] = pack2(u[2 * kk][0], u[2 * kk][1]);
    a[kk][1] = pack2(u[2 * kk][2], u[2 * kk][3]);
    a[kk][2] = pack2(u[2 * kk + 1][0], u[2 * kk + 1][1]);
    a[kk][3] = pack2(u[2 * kk + 1][2], u[2 * kk + 1][3]);
  }
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const uint16_t* wr = &W.W2[(8 * c + g) * kLpHid];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&wr[16 * kk + 2 * t]);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&wr[16 * kk + 8 + 2 * t]);
      mma16816(acc, a[kk][0], a[kk][1], a[kk][2], a[kk][3], b0, b1);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) z2[c][q] = acc[q] + W.b2[8 * c + 2 * t + (q & 1)];
  }
}

// sum over the 8 row groups (lanes with equal t)
__device__ __forceinline__ float sum_g(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 8);
  v += __shfl_xor_sync(0xffffffffu, v, 16);
  return v;
}
// sum over the 4 lanes of a row group
__device__ __forceinline__ float sum_t(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}

// Recomputes the full forward of the warp's row: layer 1, messages, layer 2
// and the output.  M must hold the node messages of every node.
struct RowFwd {
  float z1[8][4], h1[8][4], u[8][4], z2[8][4];
  float o[2], om[2], aij[2];
  int j[2];
  bool valid[2], use[2];
  float2 f[2];
};

__device__ __forceinline__ void row_forward(const SmemW& W, const LpGraph& g, const float4* node4,
                                            const float* M, const RowCtx& r, int g8, int t,
                                            RowFwd& R) {
  R.f[0] = feat_pair(g, node4, r, g8, t, R.aij[0], R.j[0]);
  R.f[1] = feat_pair(g, node4, r, g8 + 8, t, R.aij[1], R.j[1]);
  layer1(W, R.f[0], R.f[1], g8, t, R.z1, R.h1);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    R.valid[h] = slot_valid(r, g8 + 8 * h);
    bool use = false;
    if (R.valid[h]) {
      const int dij = R.j[h] - r.i;
      use = !(dij == r.nn || dij == -r.nn) && !r.dmi && !g.dmask[R.j[h]];
    }
    R.use[h] = use;
  }
  // U = bf16((H1 + M_i) + M_j)
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int col = 8 * c + 2 * t;
    float2 mi = make_float2(0.f, 0.f);
    if (r.ok) mi = *reinterpret_cast<const float2*>(&M[(size_t)r.i * kLpHid + col]);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float2 mj = make_float2(0.f, 0.f);
      if (R.valid[h]) mj = *reinterpret_cast<const float2*>(&M[(size_t)R.j[h] * kLpHid + col]);
      R.u[c][2 * h] = bfr((R.h1[c][2 * h] + mi.x) + mj.x);
      R.u[c][2 * h + 1] = bfr((R.h1[c][2 * h + 1] + mi.y) + mj.y);
    }
  }
  layer2(W, R.u, g8, t, R.z2);
  float op[2] = {0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int col = 8 * c + 2 * t;
#pragma unroll
    for (int h = 0; h < 2; ++h)
      op[h] += fmaxf(R.z2[c][2 * h], 0.f) * W.w3[col] + fmaxf(R.z2[c][2 * h + 1], 0.f) * W.w3[col + 1];
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    R.o[h] = sum_t(op[h]) + W.b3;
    R.om[h] = tanhf(R.o[h]);
  }
}

// ---- forward pass 1: node messages M_i = mean of H1 over row i ----------
__global__ void __launch_bounds__(kBlock) k_lp_fwd1(LpGraph g, const float4* node4,
                                                    const uint16_t* wbf, const float* P, float* M) {
  __shared__ SmemW W;
  load_weights(W, wbf, P);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g8 = lane >> 2, t = lane & 3;
  for (int i = blockIdx.x * kWarps + warp; i < g.n; i += gridDim.x * kWarps) {
    const RowCtx r = row_ctx(g, i);
    if (!r.ok) continue;  // warp-uniform
    float aij, z1[8][4], h1[8][4];
    int j;
    const float2 f0 = feat_pair(g, node4, r, g8, t, aij, j);
    const float2 f1 = feat_pair(g, node4, r, g8 + 8, t, aij, j);
    layer1(W, f0, f1, g8, t, z1, h1);
    const bool v0 = slot_valid(r, g8), v1 = slot_valid(r, g8 + 8);
    const float rdeg = r.len > 1 ? 1.0f / (float)(r.len - 1) : 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float s0 = sum_g((v0 ? h1[c][0] : 0.f) + (v1 ? h1[c][2] : 0.f));
      const float s1 = sum_g((v0 ? h1[c][1] : 0.f) + (v1 ? h1[c][3] : 0.f));
      if (g8 == 0)
        *reinterpret_cast<float2*>(&M[(size_t)i * kLpHid + 8 * c + 2 * t]) =
            make_float2(s0 * rdeg, s1 * rdeg);
    }
  }
}

// ---- forward pass 2: omega per slot and d' ---------------------------------
__global__ void __launch_bounds__(kBlock) k_lp_fwd2(LpGraph g, const float4* node4,
                                                    const uint16_t* wbf, const float* P,
                                                    const float* M, float* omega, float* dprime) {
  __shared__ SmemW W;
  load_weights(W, wbf, P);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g8 = lane >> 2, t = lane & 3;
  for (int i = blockIdx.x * kWarps + warp; i < g.n; i += gridDim.x * kWarps) {
    const RowCtx r = row_ctx(g, i);
    if (!r.ok) continue;
    RowFwd R;
    row_forward(W, g, node4, M, r, g8, t, R);
    float comp = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = g8 + 8 * h;
      const float w = R.use[h] ? R.om[h] : 0.f;
      if (t == 0 && row < r.len) omega[r.s0 + row] = w;
      comp += w * R.aij[h];
    }
    comp = sum_g(comp);
    if (lane == 0) dprime[i] = r.dmi ? 1.0f : g.vals[r.sd] + comp;
  }
}

// d' from stored omega and the current matrix values
__global__ void k_lp_apply_omega(LpGraph g, const float* omega, float* dprime) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n || !g.active[g.mem[i]]) return;
  if (g.dmask[i]) {
    dprime[i] = 1.0f;
    return;
  }
  float comp = 0.f;
  for (int s = g.rowptr[i]; s < g.rowptr[i + 1]; ++s) comp += omega[s] * g.vals[s];
  dprime[i] = g.vals[g.diag[i]] + comp;
}

// ---- column-line factor and solves ------------------------------------------
__global__ void k_lp_line_factor(LpGraph g, LpColumns c, const int32_t* down, const float* dprime,
                                 float* pinv, float* cdn, double* msc) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.ncol) return;
  const int m = c.mem[q];
  if (!g.active[m]) return;
  const int st = c.stride[q], nl = c.nl[q];
  float pp = 1.0f, cp = 0.0f;
  bool bad = false;
  for (int k = 0; k < nl; ++k) {
    const int i = c.top[q] + k * st;
    const bool di = g.dmask[i] != 0;
    const float a = di ? 1.0f : dprime[i];
    const float p = a - cp * cp / pp;
    if (!(p > 0.0f) || !isfinite(p)) bad = true;
    pinv[i] = 1.0f / p;
    float cc = 0.0f;
    if (k + 1 < nl && !di && !g.dmask[i + st] && down[i] >= 0) cc = g.vals[down[i]];
    cdn[i] = cc;
    pp = p;
    cp = cc;
  }
  if (bad && msc) msc[(size_t)m * 8 + 6] = 1.0;
}

// z = T'^-1 r along every column (z may alias nothing; forward sweep stored
// in z then overwritten by the backward sweep)
__global__ void k_lp_line_solve(LpGraph g, LpColumns c, const float* pinv, const float* cdn,
                                const float* r, float* z) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.ncol) return;
  if (!g.active[c.mem[q]]) return;
  const int st = c.stride[q], nl = c.nl[q], top = c.top[q];
  float yp = 0.f;
  for (int k = 0; k < nl; ++k) {
    const int i = top + k * st;
    const float yk = r[i] - (k > 0 ? cdn[i - st] * yp * pinv[i - st] : 0.f);
    z[i] = yk;
    yp = yk;
  }
  float zn = 0.f;
  for (int k = nl - 1; k >= 0; --k) {
    const int i = top + k * st;
    const float zk = (z[i] - cdn[i] * zn) * pinv[i];
    z[i] = zk;
    zn = zk;
  }
}

// per-member dots p_k . q_k for all pairs (den), slot msc[m*8 + k]
__global__ void k_lp_den(LpGraph g, const float* P, const float* Q, double* msc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int m = g.mem[i];
  if (!g.active[m]) return;
#pragma unroll
  for (int k = 0; k < kLpPairs; ++k) {
    const float v = P[(size_t)k * g.n + i] * Q[(size_t)k * g.n + i];
    if (v != 0.0f) atomicAdd(&msc[(size_t)m * 8 + k], (double)v);
  }
}

// t0 = y - p ; t1 = A t0 (Dirichlet rows identity); loss_m += t0.t1/(den K)
__global__ void k_lp_resid_energy(LpGraph g, const float* y, const float* p, float* t0,
                                  int k, double* msc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n || !g.active[g.mem[i]]) return;
  t0[i] = y[i] - p[i];
  (void)k;
  (void)msc;
}
__global__ void k_lp_spmv_energy(LpGraph g, const float* x, float* y, int k, double* msc) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
  const int lane = threadIdx.x & 15;
  float s = 0.f;
  bool ok = row < g.n;
  int m = 0;
  if (ok) {
    m = g.mem[row];
    ok = g.active[m] != 0;
  }
  if (ok) {
    const int s0 = g.rowptr[row] + lane;
    if (s0 < g.rowptr[row + 1]) s = g.vals[s0] * x[g.cols[s0]];
  }
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (ok && lane == 0) {
    const float yi = g.dmask[row] ? x[row] : s;
    y[row] = yi;
    const double den = msc[(size_t)m * 8 + k], np = msc[(size_t)m * 8 + 5];
    if (den > 0.0 && np > 0.0 && msc[(size_t)m * 8 + 6] == 0.0)
      atomicAdd(&msc[(size_t)m * 8 + 4], (double)(x[row] * yi) / (den * np));
  }
}
// u = 2 A delta / (den K) (in place on t1), scaled by 1/B (members in batch)
__global__ void k_lp_u(LpGraph g, float* t1, int k, const double* msc, float inv_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int m = g.mem[i];
  if (!g.active[m]) return;
  const double den = msc[(size_t)m * 8 + k], np = msc[(size_t)m * 8 + 5];
  const bool ok = den > 0.0 && np > 0.0 && msc[(size_t)m * 8 + 6] == 0.0;
  t1[i] = ok ? (float)(2.0 * (double)t1[i] / (den * np)) * inv_b : 0.0f;
}
// dd -= gvec * y (Dirichlet rows 0)
__global__ void k_lp_dd(LpGraph g, const float* gv, const float* y, float* dd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n || !g.active[g.mem[i]]) return;
  if (!g.dmask[i]) dd[i] -= gv[i] * y[i];
}
// number of usable pairs per member (den > 0) into msc[m*8+5]
__global__ void k_lp_count(int nmem, const uint8_t* active, double* msc) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem || !active[m]) return;
  double c = 0.0;
  for (int k = 0; k < kLpPairs; ++k) c += msc[(size_t)m * 8 + k] > 0.0 ? 1.0 : 0.0;
  msc[(size_t)m * 8 + 5] = c;
}

// ---- backward 1: output layer, layer 2, dU per slot, gradients of W2, b2,
// w3, b3 -------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_lp_bwd1(LpGraph g, const float4* node4,
                                                    const uint16_t* wbf, const float* P,
                                                    const float* M, const float* dd,
                                                    const double* msc, float* dU, float* G) {
  __shared__ SmemW W;
  __shared__ uint16_t sDZ[kWarps][16][kLpHid];
  __shared__ uint16_t sU[kWarps][16][kLpHid];
  load_weights(W, wbf, P);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g8 = lane >> 2, t = lane & 3;
  float gW2[8][4], gw3[8][2], gb2[8][2], gb3 = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    gW2[c][0] = gW2[c][1] = gW2[c][2] = gW2[c][3] = 0.f;
    gw3[c][0] = gw3[c][1] = gb2[c][0] = gb2[c][1] = 0.f;
  }
  const int ngroups = (g.n + kWarps - 1) / kWarps;
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int i = grp * kWarps + warp;
    RowCtx r = row_ctx(g, i);
    if (r.ok && msc[(size_t)r.m * 8 + 6] != 0.0) r.ok = false;  // member with a bad factor
    float dz[8][4];
    float u[8][4];
    if (r.ok) {
      RowFwd R;
      row_forward(W, g, node4, M, r, g8, t, R);
      const float ddi = dd[i];
      float dov[2];
#pragma unroll
      for (int h = 0; h < 2; ++h)
        dov[h] = R.use[h] ? ddi * R.aij[h] * (1.0f - R.om[h] * R.om[h]) : 0.f;
      if (t == 0) gb3 += dov[0] + dov[1];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int col = 8 * c + 2 * t;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int h = q >> 1;
          const float z = R.z2[c][q];
          gw3[c][q & 1] += dov[h] * fmaxf(z, 0.f);
          dz[c][q] = bfr(z > 0.f ? dov[h] * W.w3[col + (q & 1)] : 0.f);
          gb2[c][q & 1] += dz[c][q];
          u[c][q] = R.valid[h] ? R.u[c][q] : 0.f;
        }
      }
      // dU = dZ2 W2 (B operand = W2^T rows)
      uint32_t a[4][4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        a[kk][0] = pack2(dz[2 * kk][0], dz[2 * kk][1]);
        a[kk][1] = pack2(dz[2 * kk][2], dz[2 * kk][3]);
        a[kk][2] = pack2(dz[2 * kk + 1][0], dz[2 * kk + 1][1]);
        a[kk][3] = pack2(dz[2 * kk + 1][2], dz[2 * kk + 1][3]);
      }
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const uint16_t* wr = &W.W2t[(8 * c + g8) * kLpHid];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&wr[16 * kk + 2 * t]);
          const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&wr[16 * kk + 8 + 2 * t]);
          mma16816(acc, a[kk][0], a[kk][1], a[kk][2], a[kk][3], b0, b1);
        }
        const int col = 8 * c + 2 * t;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (R.valid[h])
            *reinterpret_cast<float2*>(&dU[(size_t)(r.s0 + g8 + 8 * h) * kLpHid + col]) =
                make_float2(acc[2 * h], acc[2 * h + 1]);
      }
    } else {
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int q = 0; q < 4; ++q) dz[c][q] = u[c][q] = 0.f;
    }
    // stage dZ2 and U tiles
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int col = 8 * c + 2 * t;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = g8 + 8 * h;
        sDZ[warp][row][col] = bfbits(dz[c][2 * h]);
        sDZ[warp][row][col + 1] = bfbits(dz[c][2 * h + 1]);
        sU[warp][row][col] = bfbits(u[c][2 * h]);
        sU[warp][row][col + 1] = bfbits(u[c][2 * h + 1]);
      }
    }
    __syncthreads();
    // gW2[16*warp.., :] += sum over the 64 staged slots of dZ2^T U
    const int ch = 16 * warp + g8;
#pragma unroll
    for (int kt = 0; kt < kWarps; ++kt) {
      const uint32_t a0 = pack_raw(sDZ[kt][2 * t][ch], sDZ[kt][2 * t + 1][ch]);
      const uint32_t a1 = pack_raw(sDZ[kt][2 * t][ch + 8], sDZ[kt][2 * t + 1][ch + 8]);
      const uint32_t a2 = pack_raw(sDZ[kt][2 * t + 8][ch], sDZ[kt][2 * t + 9][ch]);
      const uint32_t a3 = pack_raw(sDZ[kt][2 * t + 8][ch + 8], sDZ[kt][2 * t + 9][ch + 8]);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int n = 8 * c + g8;
        const uint32_t b0 = pack_raw(sU[kt][2 * t][n], sU[kt][2 * t + 1][n]);
        const uint32_t b1 = pack_raw(sU[kt][2 * t + 8][n], sU[kt][2 * t + 9][n]);
        mma16816(gW2[c], a0, a1, a2, a3, b0, b1);
      }
    }
    __syncthreads();
  }
  // flush the per-thread partial gradients
  const int ch = 16 * warp + g8;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int col = 8 * c + 2 * t;
    atomicAdd(&G[kLpOffW2 + ch * kLpHid + col], gW2[c][0]);
    atomicAdd(&G[kLpOffW2 + ch * kLpHid + col + 1], gW2[c][1]);
    atomicAdd(&G[kLpOffW2 + (ch + 8) * kLpHid + col], gW2[c][2]);
    atomicAdd(&G[kLpOffW2 + (ch + 8) * kLpHid + col + 1], gW2[c][3]);
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float a = sum_g(gw3[c][e]), b = sum_g(gb2[c][e]);
      if (g8 == 0) {
        atomicAdd(&G[kLpOffW3 + col + e], a);
        atomicAdd(&G[kLpOffB2 + col + e], b);
      }
    }
  }
  float s = gb3;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) atomicAdd(&G[kLpOffB3], s);
}

// ---- backward 2: messages, layer 1, gradients of W1, b1 -----------------------
__global__ void __launch_bounds__(kBlock) k_lp_bwd2(LpGraph g, const float4* node4,
                                                    const uint16_t* wbf, const float* P,
                                                    const int32_t* tslot, const double* msc,
                                                    const float* dU, float* G) {
  __shared__ SmemW W;
  __shared__ uint16_t sDZ[kWarps][16][kLpHid];
  __shared__ uint16_t sF[kWarps][16][kLpNF];
  load_weights(W, wbf, P);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g8 = lane >> 2, t = lane & 3;
  float gW1[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  float gb1[8][2];
#pragma unroll
  for (int c = 0; c < 8; ++c) gb1[c][0] = gb1[c][1] = 0.f;
  const int ngroups = (g.n + kWarps - 1) / kWarps;
  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int i = grp * kWarps + warp;
    RowCtx r = row_ctx(g, i);
    if (r.ok && msc[(size_t)r.m * 8 + 6] != 0.0) r.ok = false;
    float dz[8][4];
    float2 f[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    if (r.ok) {
      float aij, z1[8][4], h1[8][4];
      int j;
      f[0] = feat_pair(g, node4, r, g8, t, aij, j);
      f[1] = feat_pair(g, node4, r, g8 + 8, t, aij, j);
      layer1(W, f[0], f[1], g8, t, z1, h1);
      const bool v[2] = {slot_valid(r, g8), slot_valid(r, g8 + 8)};
      const float rdeg = r.len > 1 ? 1.0f / (float)(r.len - 1) : 0.0f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int col = 8 * c + 2 * t;
        float2 du[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        float dsum0 = 0.f, dsum1 = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!v[h]) continue;
          const int s = r.s0 + g8 + 8 * h;
          du[h] = *reinterpret_cast<const float2*>(&dU[(size_t)s * kLpHid + col]);
          const float2 dt = *reinterpret_cast<const float2*>(&dU[(size_t)tslot[s] * kLpHid + col]);
          dsum0 += du[h].x + dt.x;
          dsum1 += du[h].y + dt.y;
        }
        const float D0 = sum_g(dsum0) * rdeg, D1 = sum_g(dsum1) * rdeg;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float dh0 = v[h] ? du[h].x + D0 : 0.f;
          const float dh1 = v[h] ? du[h].y + D1 : 0.f;
          dz[c][2 * h] = bfr(z1[c][2 * h] > 0.f ? dh0 : 0.f);
          dz[c][2 * h + 1] = bfr(z1[c][2 * h + 1] > 0.f ? dh1 : 0.f);
          gb1[c][0] += dz[c][2 * h];
          gb1[c][1] += dz[c][2 * h + 1];
        }
      }
      if (!v[0]) f[0] = make_float2(0.f, 0.f);
      if (!v[1]) f[1] = make_float2(0.f, 0.f);
    } else {
#pragma unroll
      for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int q = 0; q < 4; ++q) dz[c][q] = 0.f;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int col = 8 * c + 2 * t;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        sDZ[warp][g8 + 8 * h][col] = bfbits(dz[c][2 * h]);
        sDZ[warp][g8 + 8 * h][col + 1] = bfbits(dz[c][2 * h + 1]);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      sF[warp][g8 + 8 * h][2 * t] = bfbits(f[h].x);
      sF[warp][g8 + 8 * h][2 * t + 1] = bfbits(f[h].y);
      sF[warp][g8 + 8 * h][2 * t + 8] = 0;
      sF[warp][g8 + 8 * h][2 * t + 9] = 0;
    }
    __syncthreads();
    const int ch = 16 * warp + g8;
#pragma unroll
    for (int kt = 0; kt < kWarps; ++kt) {
      const uint32_t a0 = pack_raw(sDZ[kt][2 * t][ch], sDZ[kt][2 * t + 1][ch]);
      const uint32_t a1 = pack_raw(sDZ[kt][2 * t][ch + 8], sDZ[kt][2 * t + 1][ch + 8]);
      const uint32_t a2 = pack_raw(sDZ[kt][2 * t + 8][ch], sDZ[kt][2 * t + 9][ch]);
      const uint32_t a3 = pack_raw(sDZ[kt][2 * t + 8][ch + 8], sDZ[kt][2 * t + 9][ch + 8]);
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int n = 8 * c + g8;
        const uint32_t b0 = pack_raw(sF[kt][2 * t][n], sF[kt][2 * t + 1][n]);
        const uint32_t b1 = pack_raw(sF[kt][2 * t + 8][n], sF[kt][2 * t + 9][n]);
        mma16816(gW1[c], a0, a1, a2, a3, b0, b1);
      }
    }
    __syncthreads();
  }
  const int ch = 16 * warp + g8;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int col = 8 * c + 2 * t;
    atomicAdd(&G[kLpOffW1 + ch * kLpNF + col], gW1[c][0]);
    atomicAdd(&G[kLpOffW1 + ch * kLpNF + col + 1], gW1[c][1]);
    atomicAdd(&G[kLpOffW1 + (ch + 8) * kLpNF + col], gW1[c][2]);
    atomicAdd(&G[kLpOffW1 + (ch + 8) * kLpNF + col + 1], gW1[c][3]);
  }
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int col = 8 * c + 2 * t;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float b = sum_g(gb1[c][e]);
      if (g8 == 0) atomicAdd(&G[kLpOffB1 + col + e], b);
    }
  }
}

// ---- Adam and the bf16 weight copies -----------------------------------------
__global__ void k_lp_adam(int np, float* p, const float* gr, float* m, float* v, float lr,
                          float bc1, float bc2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  const float gq = gr[q];
  const float mq = 0.9f * m[q] + 0.1f * gq;
  const float vq = 0.999f * v[q] + 0.001f * gq * gq;
  m[q] = mq;
  v[q] = vq;
  p[q] -= lr * (mq / bc1) / (sqrtf(vq / bc2) + 1e-8f);
}

__global__ void k_lp_refresh(const float* P, uint16_t* wbf) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int nW1 = kLpHid * kLpNF, nW2 = kLpHid * kLpHid;
  if (q < nW1) wbf[q] = bfbits(P[kLpOffW1 + q]);
  if (q < nW2) {
    wbf[nW1 + q] = bfbits(P[kLpOffW2 + q]);
    const int r = q / kLpHid, c = q % kLpHid;  // W2t[c][r] = W2[r][c]
    wbf[nW1 + nW2 + c * kLpHid + r] = bfbits(P[kLpOffW2 + q]);
  }
}

int grid_rows(long n) {
  long b = (n + kWarps - 1) / kWarps;
  const long cap = 152L * 16;
  return (int)std::max(1L, std::min(b, cap));
}
inline int cdivl(long a, long b) { return (int)((a + b - 1) / b); }

void lp_forward_impl(const LpModel& m, const LpGraph& g, LpWork& w, cudaStream_t st) {
  k_lp_nodes<<<cdivl(g.n, 256), 256, 0, st>>>(g, w.node4);
  k_lp_fwd1<<<grid_rows(g.n), kBlock, 0, st>>>(g, w.node4, m.wbf, m.params, w.M);
  k_lp_fwd2<<<grid_rows(g.n), kBlock, 0, st>>>(g, w.node4, m.wbf, m.params, w.M, w.omega,
                                               w.dprime);
  CG_TRY(cudaPeekAtLastError());
}

// loss and dL/dd' into w.dd; returns nothing (scalars stay in w.msc)
void lp_loss_dd(const LpGraph& g, const LpColumns& c, const int32_t* down, LpWork& w,
                const float* P, const float* Q, cudaStream_t st, double* loss, int* nused) {
  CG_TRY(cudaMemsetAsync(w.msc, 0, sizeof(double) * 8 * w.nmem, st));
  CG_TRY(cudaMemsetAsync(w.dd, 0, sizeof(float) * g.n, st));
  k_lp_line_factor<<<cdivl(c.ncol, 128), 128, 0, st>>>(g, c, down, w.dprime, w.piv, w.cdn, w.msc);
  k_lp_den<<<cdivl(g.n, 256), 256, 0, st>>>(g, P, Q, w.msc);
  k_lp_count<<<cdivl(w.nmem, 128), 128, 0, st>>>(w.nmem, g.active, w.msc);
  std::vector<double> h((size_t)8 * w.nmem);
  CG_TRY(cudaMemcpyAsync(h.data(), w.msc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  CG_TRY(cudaStreamSynchronize(st));
  int b = 0;
  for (int m = 0; m < w.nmem; ++m)
    if (h[(size_t)m * 8 + 5] > 0.0 && h[(size_t)m * 8 + 6] == 0.0) ++b;
  const float inv_b = b > 0 ? 1.0f / (float)b : 0.0f;
  for (int k = 0; k < kLpPairs; ++k) {
    const float* pk = P + (size_t)k * g.n;
    const float* qk = Q + (size_t)k * g.n;
    float* yk = w.y + (size_t)k * g.n;
    k_lp_line_solve<<<cdivl(c.ncol, 128), 128, 0, st>>>(g, c, w.piv, w.cdn, qk, yk);
    k_lp_resid_energy<<<cdivl(g.n, 256), 256, 0, st>>>(g, yk, pk, w.t0, k, w.msc);
    k_lp_spmv_energy<<<cdivl((long)g.n * 16, 256), 256, 0, st>>>(g, w.t0, w.t1, k, w.msc);
    k_lp_u<<<cdivl(g.n, 256), 256, 0, st>>>(g, w.t1, k, w.msc, inv_b);
    k_lp_line_solve<<<cdivl(c.ncol, 128), 128, 0, st>>>(g, c, w.piv, w.cdn, w.t1, w.t0);
    k_lp_dd<<<cdivl(g.n, 256), 256, 0, st>>>(g, w.t0, yk, w.dd);
  }
  CG_TRY(cudaPeekAtLastError());
  CG_TRY(cudaMemcpyAsync(h.data(), w.msc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  CG_TRY(cudaStreamSynchronize(st));
  double L = 0.0;
  for (int m = 0; m < w.nmem; ++m)
    if (h[(size_t)m * 8 + 5] > 0.0 && h[(size_t)m * 8 + 6] == 0.0) L += h[(size_t)m * 8 + 4];
  if (loss) *loss = b > 0 ? L / b : 0.0;
  if (nused) *nused = b;
}

void lp_backward(LpModel& m, const LpGraph& g, const int32_t* tslot, LpWork& w, cudaStream_t st) {
  CG_TRY(cudaMemsetAsync(m.grads, 0, sizeof(float) * kLpParams, st));
  k_lp_bwd1<<<grid_rows(g.n), kBlock, 0, st>>>(g, w.node4, m.wbf, m.params, w.M, w.dd, w.msc,
                                               w.dU, m.grads);
  k_lp_bwd2<<<grid_rows(g.n), kBlock, 0, st>>>(g, w.node4, m.wbf, m.params, tslot, w.msc, w.dU,
                                               m.grads);
  CG_TRY(cudaPeekAtLastError());
}

}  // namespace

// ---- host API -----------------------------------------------------------------
void lp_alloc(LpModel& m) {
  CG_TRY(cudaMalloc((void**)&m.params, sizeof(float) * kLpParams));
  CG_TRY(cudaMalloc((void**)&m.grads, sizeof(float) * kLpParams));
  CG_TRY(cudaMalloc((void**)&m.adam_m, sizeof(float) * kLpParams));
  CG_TRY(cudaMalloc((void**)&m.adam_v, sizeof(float) * kLpParams));
  CG_TRY(cudaMalloc((void**)&m.wbf, sizeof(uint16_t) * (kLpHid * kLpNF + 2 * kLpHid * kLpHid)));
  CG_TRY(cudaMemset(m.adam_m, 0, sizeof(float) * kLpParams));
  CG_TRY(cudaMemset(m.adam_v, 0, sizeof(float) * kLpParams));
  m.steps = 0;
}
void lp_free(LpModel& m) {
  cudaFree(m.params); cudaFree(m.grads); cudaFree(m.adam_m); cudaFree(m.adam_v); cudaFree(m.wbf);
  m.params = m.grads = m.adam_m = m.adam_v = nullptr;
  m.wbf = nullptr;
}
void lp_refresh(LpModel& m, cudaStream_t st) {
  k_lp_refresh<<<cdivl(kLpHid * kLpHid, 256), 256, 0, st>>>(m.params, m.wbf);
  CG_TRY(cudaPeekAtLastError());
}
void lp_set_params(LpModel& m, const float* host, cudaStream_t st) {
  CG_TRY(cudaMemcpyAsync(m.params, host, sizeof(float) * kLpParams, cudaMemcpyHostToDevice, st));
  lp_refresh(m, st);
  CG_TRY(cudaStreamSynchronize(st));
}
void lp_get_params(const LpModel& m, float* host, cudaStream_t st) {
  CG_TRY(cudaMemcpyAsync(host, m.params, sizeof(float) * kLpParams, cudaMemcpyDeviceToHost, st));
  CG_TRY(cudaStreamSynchronize(st));
}

void lp_work_alloc(LpWork& w, long n, long nnz, int nmem, bool training) {
  lp_work_free(w);
  w.n = n; w.nnz = nnz; w.nmem = nmem; w.training = training;
  CG_TRY(cudaMalloc((void**)&w.node4, sizeof(float4) * n));
  CG_TRY(cudaMalloc((void**)&w.M, sizeof(float) * n * kLpHid));
  CG_TRY(cudaMalloc((void**)&w.omega, sizeof(float) * nnz));
  CG_TRY(cudaMemset(w.omega, 0, sizeof(float) * nnz));
  CG_TRY(cudaMalloc((void**)&w.dprime, sizeof(float) * n));
  CG_TRY(cudaMalloc((void**)&w.msc, sizeof(double) * 8 * std::max(nmem, 1)));
  CG_TRY(cudaMemset(w.msc, 0, sizeof(double) * 8 * std::max(nmem, 1)));
  if (training) {
    CG_TRY(cudaMalloc((void**)&w.dU, sizeof(float) * nnz * kLpHid));
    CG_TRY(cudaMalloc((void**)&w.dd, sizeof(float) * n));
    CG_TRY(cudaMalloc((void**)&w.piv, sizeof(float) * n));
    CG_TRY(cudaMalloc((void**)&w.cdn, sizeof(float) * n));
    CG_TRY(cudaMalloc((void**)&w.y, sizeof(float) * n * kLpPairs));
    CG_TRY(cudaMalloc((void**)&w.t0, sizeof(float) * n));
    CG_TRY(cudaMalloc((void**)&w.t1, sizeof(float) * n));
  }
}
void lp_work_free(LpWork& w) {
  float** fs[] = {&w.M, &w.dU, &w.omega, &w.dprime, &w.dd, &w.piv, &w.cdn, &w.y, &w.t0, &w.t1};
  for (float** p : fs) { if (*p) cudaFree(*p); *p = nullptr; }
  if (w.node4) cudaFree(w.node4);
  w.node4 = nullptr;
  if (w.msc) cudaFree(w.msc);
  w.msc = nullptr;
}

void lp_forward(const LpModel& m, const LpGraph& g, LpWork& w, cudaStream_t st) {
  lp_forward_impl(m, g, w, st);
}

void lp_apply_omega(const LpGraph& g, LpWork& w, cudaStream_t st) {
  k_lp_apply_omega<<<cdivl(g.n, 256), 256, 0, st>>>(g, w.omega, w.dprime);
  CG_TRY(cudaPeekAtLastError());
}

void lp_loss_grad(LpModel& m, const LpGraph& g, const LpColumns& c, const int32_t* down,
                  const int32_t* tslot, LpWork& w, const float* P, const float* Q,
                  cudaStream_t st, double* loss, int* nused) {
  lp_forward_impl(m, g, w, st);
  lp_loss_dd(g, c, down, w, P, Q, st, loss, nused);
  lp_backward(m, g, tslot, w, st);
}

void lp_train_step(LpModel& m, const LpGraph& g, const LpColumns& c, const int32_t* down,
                   const int32_t* tslot, LpWork& w, const float* P, const float* Q,
                   cudaStream_t st, double* loss, int* nused) {
  int b = 0;
  lp_loss_grad(m, g, c, down, tslot, w, P, Q, st, loss, &b);
  if (nused) *nused = b;
  if (b == 0) return;
  if (loss) m.last_loss = *loss;
  m.steps += 1;
  const float bc1 = 1.0f - powf(0.9f, (float)m.steps);
  const float bc2 = 1.0f - powf(0.999f, (float)m.steps);
  k_lp_adam<<<cdivl(kLpParams, 256), 256, 0, st>>>(kLpParams, m.params, m.grads, m.adam_m,
                                                    m.adam_v, (float)m.lr, bc1, bc2);
  lp_refresh(m, st);
}

}  // namespace cathy

#define CATHY_TRY(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) throw cathy::CudaError(_e, #expr); } while (0)
// ---- C ABI: standalone model handle (training on caller graphs, checks) -----
namespace {
struct LpHandle {
  cathy::LpModel m;
  cudaStream_t st = nullptr;
  int device = 0;
};

template <class F>
int lp_guard(F&& f) {
  try {
    return f();
  } catch (const cathy::CudaError& e) {
    fprintf(stderr, "cathy_gb300_lp: CUDA error %s in %s\n", cudaGetErrorString(e.err),
            e.what.c_str());
    return CATHY_GB300_ENODEV;
  } catch (const std::string& s) {
    fprintf(stderr, "cathy_gb300_lp: %s\n", s.c_str());
    return CATHY_GB300_EINVAL;
  }
}
}  // namespace

namespace cathy {
LpModel* lp_model_of(void* handle) { return handle ? &((LpHandle*)handle)->m : nullptr; }
}  // namespace cathy

extern "C" {

int32_t cathy_gb300_lp_create(const float* params, int32_t device, void** model) {
  if (!model) return CATHY_GB300_EINVAL;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) return CATHY_GB300_ENODEV;
  return lp_guard([&]() {
    LpHandle* h = new LpHandle();
    h->device = device;
    CATHY_TRY(cudaSetDevice(device));
    CATHY_TRY(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    cathy::lp_alloc(h->m);
    std::vector<float> p(cathy::kLpParams, 0.0f);
    if (params) std::copy(params, params + cathy::kLpParams, p.begin());
    cathy::lp_set_params(h->m, p.data(), h->st);
    *model = h;
    return CATHY_GB300_OK;
  });
}

int32_t cathy_gb300_lp_destroy(void* model) {
  if (!model) return CATHY_GB300_EINVAL;
  LpHandle* h = (LpHandle*)model;
  cudaSetDevice(h->device);
  cathy::lp_free(h->m);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return CATHY_GB300_OK;
}

int32_t cathy_gb300_lp_params(void* model, float* get, const float* set, double lr,
                              int64_t* steps) {
  if (!model) return CATHY_GB300_EINVAL;
  LpHandle* h = (LpHandle*)model;
  return lp_guard([&]() {
    CATHY_TRY(cudaSetDevice(h->device));
    if (set) cathy::lp_set_params(h->m, set, h->st);
    if (get) cathy::lp_get_params(h->m, get, h->st);
    if (lr > 0.0) h->m.lr = lr;
    if (steps) *steps = h->m.steps;
    return CATHY_GB300_OK;
  });
}

int32_t cathy_gb300_lp_eval(void* model, int32_t n, int32_t nnod, const int32_t* rowptr,
                            const int32_t* cols, const float* vals, const uint8_t* dmask,
                            const float* ks, const float* pnodi, const float* et2, float dt,
                            int32_t npairs, const float* P, const float* Q, int32_t train_steps,
                            double* loss, float* dprime, float* omega, float* grads) {
  using namespace cathy;
  if (!model || n <= 0 || nnod <= 0 || n % nnod != 0 || !rowptr || !cols || !vals || !dmask ||
      !ks || !pnodi || !et2 || npairs < 0 || npairs > kLpPairs || (npairs && (!P || !Q)) ||
      train_steps < 0)
    return CATHY_GB300_EINVAL;
  LpHandle* h = (LpHandle*)model;
  return lp_guard([&]() {
    CATHY_TRY(cudaSetDevice(h->device));
    cudaStream_t st = h->st;
    const long nnz = rowptr[n];
    std::vector<int32_t> diag(n, -1), down(n, -1), tslot(nnz), mem(n, 0);
    for (int i = 0; i < n; ++i) {
      if (rowptr[i + 1] - rowptr[i] > 16) throw std::string("matrix row longer than 16 entries");
      for (int s = rowptr[i]; s < rowptr[i + 1]; ++s) {
        const int j = cols[s];
        if (j == i) diag[i] = s;
        if (j == i + nnod) down[i] = s;
        int t = -1;
        for (int q = rowptr[j]; q < rowptr[j + 1]; ++q)
          if (cols[q] == i) t = q;
        if (t < 0) throw std::string("pattern is not structurally symmetric");
        tslot[s] = t;
      }
      if (diag[i] < 0) throw std::string("row without diagonal");
    }
    const int ncol = nnod, nl = n / nnod;
    std::vector<int32_t> ctop(ncol), cstride(ncol, nnod), cnl(ncol, nl), cmem(ncol, 0);
    for (int c = 0; c < ncol; ++c) ctop[c] = c;
    DBuf<int32_t> d_rowptr, d_cols, d_diag, d_down, d_tslot, d_mem, d_nnod, d_ctop, d_cstr, d_cnl,
        d_cmem;
    DBuf<float> d_vals, d_ks, d_pn, d_et2, d_dt, d_P, d_Q;
    DBuf<uint8_t> d_dm, d_act;
    d_rowptr.alloc(n + 1); d_rowptr.upload(rowptr, n + 1, st);
    d_cols.alloc(nnz); d_cols.upload(cols, nnz, st);
    d_diag.alloc(n); d_diag.upload(diag.data(), n, st);
    d_down.alloc(n); d_down.upload(down.data(), n, st);
    d_tslot.alloc(nnz); d_tslot.upload(tslot.data(), nnz, st);
    d_mem.alloc(n); d_mem.upload(mem.data(), n, st);
    d_nnod.alloc(1); d_nnod.upload(&nnod, 1, st);
    d_ctop.alloc(ncol); d_ctop.upload(ctop.data(), ncol, st);
    d_cstr.alloc(ncol); d_cstr.upload(cstride.data(), ncol, st);
    d_cnl.alloc(ncol); d_cnl.upload(cnl.data(), ncol, st);
    d_cmem.alloc(ncol); d_cmem.upload(cmem.data(), ncol, st);
    d_vals.alloc(nnz); d_vals.upload(vals, nnz, st);
    d_ks.alloc(n); d_ks.upload(ks, n, st);
    d_pn.alloc(n); d_pn.upload(pnodi, n, st);
    d_et2.alloc(n); d_et2.upload(et2, n, st);
    d_dt.alloc(1); d_dt.upload(&dt, 1, st);
    d_dm.alloc(n); d_dm.upload(dmask, n, st);
    const uint8_t one = 1;
    d_act.alloc(1); d_act.upload(&one, 1, st);
    d_P.alloc((size_t)kLpPairs * n); d_P.zero(st);
    d_Q.alloc((size_t)kLpPairs * n); d_Q.zero(st);
    if (npairs) {
      d_P.upload(P, (size_t)npairs * n, st);
      d_Q.upload(Q, (size_t)npairs * n, st);
    }
    LpGraph g{n, d_rowptr.p, d_cols.p, d_vals.p, d_diag.p, d_dm.p, d_mem.p, d_nnod.p,
              d_ks.p, d_pn.p, d_et2.p, d_dt.p, d_act.p};
    LpColumns c{ncol, d_ctop.p, d_cstr.p, d_cnl.p, d_cmem.p};
    LpWork w;
    lp_work_alloc(w, n, nnz, 1, true);
    double L = 0.0;
    int used = 0;
    if (train_steps == 0) {
      lp_loss_grad(h->m, g, c, d_down.p, d_tslot.p, w, d_P.p, d_Q.p, st, &L, &used);
    } else {
      for (int k = 0; k < train_steps; ++k)
        lp_train_step(h->m, g, c, d_down.p, d_tslot.p, w, d_P.p, d_Q.p, st, &L, &used);
      lp_forward(h->m, g, w, st);
    }
    if (dprime) CATHY_TRY(cudaMemcpyAsync(dprime, w.dprime, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    if (omega) CATHY_TRY(cudaMemcpyAsync(omega, w.omega, sizeof(float) * nnz, cudaMemcpyDeviceToHost, st));
    if (grads) CATHY_TRY(cudaMemcpyAsync(grads, h->m.grads, sizeof(float) * kLpParams, cudaMemcpyDeviceToHost, st));
    CATHY_TRY(cudaStreamSynchronize(st));
    lp_work_free(w);
    if (loss) *loss = L;
    return CATHY_GB300_OK;
  });
}

}  // extern "C"
