// Device engine of the GB300 CATHY subsurface solver (internal header).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cathy_gb300.h"
#include "mesh.h"

namespace cathy {

#define CG_TRY(expr)                                   \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) throw CudaError(_e, #expr); \
  } while (0)

struct CudaError {
  cudaError_t err;
  std::string what;
  CudaError(cudaError_t e, const char* w) : err(e), what(w) {}
};

// A device allocation owned by the engine.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  bool owned = true;
  void alloc(size_t count) {
    free();
    n = count;
    owned = true;
    if (count) CG_TRY(cudaMalloc((void**)&p, sizeof(T) * count));
  }
  // a non-owning window into another allocation
  void view(T* ptr, size_t count) {
    free();
    p = ptr;
    n = count;
    owned = false;
  }
  void zero(cudaStream_t s) {
    if (n) CG_TRY(cudaMemsetAsync(p, 0, sizeof(T) * n, s));
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    if (count) CG_TRY(cudaMemcpyAsync(p, h, sizeof(T) * count, cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t count, cudaStream_t s) const {
    if (count) CG_TRY(cudaMemcpyAsync(h, p, sizeof(T) * count, cudaMemcpyDeviceToHost, s));
  }
  void free() {
    if (p && owned) cudaFree(p);
    p = nullptr;
    n = 0;
    owned = true;
  }
  ~DBuf() { free(); }
};

// Rows of one member split into fixed-size chunks: block b covers rows
// [r0[b], r1[b]) of member mem[b].  Per-member reductions then need one
// atomic per block.
struct BlockMap {
  int nblk = 0;
  DBuf<int32_t> mem, r0, r1;
  // 16-row map of the FP32 Picard path only: per entry the ranges of its
  // rows' incidence records [x, y) and matrix slots [z, w), and of their
  // gather-list bytes [eg.x, eg.y) (copied whole into shared memory by the
  // staged assembly)
  DBuf<int4> ent;
  DBuf<longlong2> eg;
};

class Engine;  // defined in engine.cu

Engine* engine_create(int nmembers, const cathy_member_t* members,
                      const cathy_opts_t& opts);
void engine_destroy(Engine* e);
int engine_step(Engine* e, int* nactive);
int engine_run(Engine* e, int max_steps, int* nsteps);
int engine_sizes(Engine* e, int m, int32_t* out5);
int engine_get_state(Engine* e, int m, double* pnew, double* time,
                     double* deltat, int32_t* status);
int engine_set_state(Engine* e, int m, const double* ptimep, double time,
                     double deltat);
int engine_get_saturation(Engine* e, int m, double* sw);
int engine_get_seepage(Engine* e, int m, int32_t* sfex, double* sfq);
int engine_num_records(Engine* e, int m, int32_t* ni, int32_t* ns);
int engine_get_records(Engine* e, int m, cathy_iter_rec_t* ir,
                       cathy_step_rec_t* sr);
int engine_get_mesh(Engine* e, int m, double* x, double* y, double* z,
                    int32_t* tetra, int32_t* rowptr, int32_t* cols);
int engine_picard_system(Engine* e, int m, double* vals, double* rhs,
                         double* xt5, int32_t* dirmask);
int engine_reset(Engine* e);
int engine_profile(Engine* e, int enable, double* spmv_ms, int64_t* spmv_launches,
                   double* spmv_bytes);
int engine_timers(Engine* e, double* out, int n);
int engine_attach_learned(Engine* e, void* model, int mode);
int engine_learned_stats(Engine* e, double* out, int n);
int engine_autotune(Engine* e, int nrep, int32_t* sched, double* ms);
int engine_set_schedule(Engine* e, int asm_blocks, int spmv_per_sm, int asm_staged,
                        int spmv_staged);
int engine_phase_timers(Engine* e, int enable, double* out, int n);
int engine_time_assembly(Engine* e, int nrep, double* ms, double* bytes, int64_t* rows);
int engine_stats(Engine* e, double* gpu_ms, int64_t* launches,
                 int64_t* lin_iters, int64_t* nl_iters);

// Fortran drop-ins (dropins in engine.cu)
int dropin_symslv(int n, int nterm, int numdir, const int32_t* noddir,
                  const int32_t* ja, const int32_t* topol, double* pnew,
                  const double* tnoti, const double* coef1, double* coef2,
                  int itmxcg, double tolcg, double rmin, int32_t* niter,
                  double* err, double* res);
int dropin_nsyslv(int isolv, int n, int nterm, int numdir,
                  const int32_t* noddir, const int32_t* ja,
                  const int32_t* topol, double* pnew, const double* tnoti,
                  const double* coef1, double* coef2, int itmxcg, double tolcg,
                  double rmin, int32_t* niter, double* err, double* res);
int dropin_asspic(int nt, int ntri, const int32_t* tetra, const int32_t* tetja,
                  const double* lmass, double* coef1, double* coef2,
                  double* coef4, const double* et1e, const double* pel,
                  const double* permx, const double* permy,
                  const double* permz, const double* ckrwe,
                  const double* volur, const double* volu, const double* bi,
                  const double* ci, const double* di, int maxstr, int nterm);

}  // namespace cathy
