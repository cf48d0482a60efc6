// Device kernels of the GB300 CATHY subsurface solver.
//
// Layout in HBM (all members of an ensemble concatenated):
//   nodes   : member m owns rows [node_off[m], node_off[m+1]); inside a member
//             node k*nnod + c is column c, layer k (GEN3D numbering), so the
//             first nnod rows of a member are its surface nodes.
//   elements: 4 node ids (int4, global 0-based) + one 64/128-byte record of
//             time-invariant local data (stiffness shape S, gravity g,
//             volume, volume*porosity) in the matrix value type MT.
//   matrix  : one full CSR over all members (sorted columns, int32), values
//             in MT; Dirichlet rows are masked by the operator, never edited.
// Every per-member reduction uses block maps whose blocks never straddle two
// members, so a block does one atomic per reduced quantity.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cathy {

constexpr int kGroup = 16;       // lanes per matrix row (max row length 15)
constexpr int kThreads = 256;    // threads per block
constexpr int kRowsPerBlock16 = kThreads / kGroup;
constexpr int kMaxLayers = 128;  // column-line preconditioner limit

// member action bits for one macro-iteration
enum : uint8_t {
  ACT_COMMIT = 1,     // accept the previous step: ptimep <- pnew, ...
  ACT_BACKSTEP = 2,   // restore the previous time level (bkstep.f)
  ACT_START = 4,      // new time level: atm update, switching, pold, ptnew
  ACT_NEXT = 8,       // next nonlinear iteration: pold <- pnew, ptnew
  ACT_ITER = 16,      // run one nonlinear iteration this macro-iteration
};

// per-member scalars on the device (read by kernels)
struct MemberScal {
  double deltat, time, tetaf, scf, pmin, omega, tolswi, deltat_r;
  double atm_ta, atm_tb;   // interpolation times for ATMPOT
  double atm_va, atm_vb;   // homogeneous rates (hspatm != 0)
  int32_t atm_mode;        // 0 keep, 1 interpolate, 2 constant vb
  int32_t hspatm, ieto, nlrelx;
  int32_t nnod, nstr, iopt, kslope;  // KSLOPE 0 (analytical) or 1 (chord slope)
  double tolksl;                      // chord slope once |PTNEW - PTOLD| >= TOLKSL
  float deltat_rf, tetaf_f;           // 1/DELTAT and TETAF rounded to FP32 by the host
};

// per-member reduction accumulators (zeroed before use).  RD_DSTORE_C and
// RD_STORE1_C hold the FP64 storage change and storage of the step accepted
// in the previous macro-iteration (the FP32 path forms them when the step
// is committed, see k_start_vg_f32).
enum {
  RD_DSTORE = 0, RD_NDIN, RD_NDOUT, RD_ADIN, RD_ADOUT, RD_ANIN, RD_ANOUT,
  RD_PL2, RD_FL2, RD_STORE1, RD_DSTORE_C, RD_STORE1_C,
  RD_SFFLW, RD_KSF,  // seepage faces: SFFLW and KSF of the iteration (k_extall)
  RD_NUM
};

template <class MT>
struct __align__(sizeof(MT) * 16) TetRec {
  MT S[10];   // (Kx b_k b_l + Ky c_k c_l + Kz d_k d_l) / V, k<=l packed
  MT g[4];    // Kz d_k ivol (gravity)
  MT vol;     // |V|
  MT vpel;    // |V| * element mean porosity
};

__host__ __device__ inline int sym_idx(int k, int l) {
  // packed upper index of (k,l), k,l in 0..3
  if (k > l) { int t = k; k = l; l = t; }
  return k * 4 - (k * (k - 1)) / 2 + (l - k);
}

}  // namespace cathy
