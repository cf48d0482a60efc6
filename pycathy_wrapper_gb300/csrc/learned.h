// Learned column-line preconditioner (internal header).
//
// A small edge-wise message-passing network reads the assembled Picard
// matrix and the local soil state and predicts, for every off-diagonal slot
// (i, j) that the column-line (vertical tridiagonal block Jacobi)
// preconditioner drops, a weight omega_ij in (-1, 1).  The preconditioner is
// then built on the corrected diagonal
//     d'_i = a_ii + sum_{j horizontal, not Dirichlet} omega_ij a_ij
// (a learned, per-edge signed relaxation of the row-sum compensation of
// modified incomplete factorisations; omega = 0 is the plain column-line
// factor).
//
// Network (hidden width 64, BF16 weights and activations, FP32 accumulation
// on the tensor cores through mma.sync m16n8k16):
//   f_s (16, 8 used)  -> H1 = relu(W1 f + b1)
//   M_i = mean_{s in row i} H1_s
//   U_s = H1_s + M_i + M_j -> H2 = relu(W2 U + b2) -> o = w3 . H2 + b3
//   omega = tanh(o)
// Training minimises, over Krylov pairs (p, q = A p) collected from the
// plain solver's PCG iterations, L = mean (T'^-1 q - p)^T A (T'^-1 q - p) /
// (p^T q) with hand-written backward and Adam kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cathy {

constexpr int kLpNF = 16;
constexpr int kLpHid = 64;
// packed parameter vector: W1 (64x16), b1 (64), W2 (64x64), b2 (64), w3 (64), b3 (1)
constexpr int kLpOffW1 = 0;
constexpr int kLpOffB1 = kLpOffW1 + kLpHid * kLpNF;
constexpr int kLpOffW2 = kLpOffB1 + kLpHid;
constexpr int kLpOffB2 = kLpOffW2 + kLpHid * kLpHid;
constexpr int kLpOffW3 = kLpOffB2 + kLpHid;
constexpr int kLpOffB3 = kLpOffW3 + kLpHid;
constexpr int kLpParams = kLpOffB3 + 1;  // 5313
constexpr int kLpPairs = 4;              // Krylov pairs kept per member

// Device view of a batch of member graphs (the engine's concatenated CSR).
struct LpGraph {
  int n;                        // rows (all members)
  const int32_t* rowptr;        // n+1, full CSR, sorted columns
  const int32_t* cols;
  const float* vals;            // Picard matrix (FP32)
  const int32_t* diag;          // n: slot of the diagonal
  const uint8_t* dmask;         // n: Dirichlet rows
  const int32_t* mem;           // n: member of the node
  const int32_t* nnod;          // per member: nodes per layer
  const float* ks;              // n: nodal saturated conductivity
  const float* pnodi;           // n: porosity
  const float* et2;             // n: dSw/dpsi (cap = pnodi * et2)
  const float* dt;              // per member: time step
  const uint8_t* active;        // per member: include in this pass
};

// Column structure for the line solves: column c has top node top[c] and
// nl[c] nodes spaced nnod_c apart.
struct LpColumns {
  int ncol;
  const int32_t* top;
  const int32_t* stride;        // nnod of the column's member
  const int32_t* nl;            // nodes in the column
  const int32_t* mem;           // member of the column
};

// Model: parameters, optimiser state and the bf16 copies the kernels read.
struct LpModel {
  float* params = nullptr;      // kLpParams fp32 master weights
  float* grads = nullptr;       // kLpParams
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  uint16_t* wbf = nullptr;      // bf16: W1 (64x16) | W2 (64x64) | W2^T (64x64)
  int64_t steps = 0;
  double lr = 1e-3;
  double last_loss = 0.0;
};

// The model behind a cathy_gb300_lp_create handle.
LpModel* lp_model_of(void* handle);

void lp_alloc(LpModel& m);
void lp_free(LpModel& m);
void lp_set_params(LpModel& m, const float* host, cudaStream_t st);
void lp_get_params(const LpModel& m, float* host, cudaStream_t st);
// refresh the bf16 weight copies from the fp32 master weights
void lp_refresh(LpModel& m, cudaStream_t st);

// Workspace sized for a graph of n rows and nnz slots.
struct LpWork {
  long n = 0, nnz = 0;
  float4* node4 = nullptr;      // n: per-node feature inputs
  float* M = nullptr;           // n x 64 node messages
  float* dU = nullptr;          // nnz x 64 (training only)
  float* omega = nullptr;       // nnz: per-slot weights (0 on unused slots)
  float* dprime = nullptr;      // n: corrected diagonal
  float* dd = nullptr;          // n: dL/dd'
  float* piv = nullptr;         // n: line pivots (1/pivot)
  float* cdn = nullptr;         // n: vertical coupling to the node below
  float* y = nullptr;           // kLpPairs x n
  float* t0 = nullptr;          // n scratch
  float* t1 = nullptr;          // n scratch
  double* msc = nullptr;        // per member scalars (den[k], loss, count)
  int nmem = 0;
  bool training = false;
};
void lp_work_alloc(LpWork& w, long n, long nnz, int nmem, bool training);
void lp_work_free(LpWork& w);

// Inference: omega per slot and the corrected diagonal d' for the members
// flagged in g.active (rows of other members are untouched).
void lp_forward(const LpModel& m, const LpGraph& g, LpWork& w, cudaStream_t st);
// d' from stored omega and the current matrix (cheap refresh between
// network evaluations)
void lp_apply_omega(const LpGraph& g, LpWork& w, cudaStream_t st);

// One training step on the batch: loss and dL/dd' from the Krylov pairs
// (p_k, q_k), k < kLpPairs, stored as kLpPairs x n arrays; backward through
// the network; Adam update.  Returns the batch loss (mean over members with
// at least one usable pair) through *loss (host, synchronises).
// `down` is the slot of (i, i+nnod) per row (-1 if none); `tslot` the
// transposed slot of every CSR slot.
void lp_train_step(LpModel& m, const LpGraph& g, const LpColumns& c, const int32_t* down,
                   const int32_t* tslot, LpWork& w, const float* P, const float* Q,
                   cudaStream_t st, double* loss, int* nmembers_used);

// Loss and parameter gradients (into m.grads) without an update.
void lp_loss_grad(LpModel& m, const LpGraph& g, const LpColumns& c, const int32_t* down,
                  const int32_t* tslot, LpWork& w, const float* P, const float* Q,
                  cudaStream_t st, double* loss, int* nmembers_used);

}  // namespace cathy
