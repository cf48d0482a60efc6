// extern "C" entry points of libcathy_gb300 (declared in include/cathy_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>

#include "engine.h"

using namespace cathy;

namespace {
int g_last_verbose = 0;

int have_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const CudaError& e) {
    fprintf(stderr, "cathy_gb300: CUDA error %s in %s\n", cudaGetErrorString(e.err), e.what.c_str());
    return CATHY_GB300_ENODEV;
  } catch (const std::string& s) {
    fprintf(stderr, "cathy_gb300: %s\n", s.c_str());
    return CATHY_GB300_EINVAL;
  } catch (const std::bad_alloc&) {
    return CATHY_GB300_ENOMEM;
  }
}
}  // namespace

extern "C" {

int32_t cathy_gb300_version(void) { return 100; }

int32_t cathy_gb300_device_count(void) { return have_device(); }

int32_t cathy_gb300_mesh(const cathy_dem_t* dem, int32_t iopt, int32_t* out5,
                         double* x, double* y, double* z, int32_t* tetra,
                         int32_t* rowptr, int32_t* cols) {
  if (!dem || !out5 || (iopt != 1 && iopt != 2)) return CATHY_GB300_EINVAL;
  HostMesh m;
  if (!build_mesh(*dem, iopt, m)) return CATHY_GB300_EMESH;
  out5[0] = m.n; out5[1] = m.nt; out5[2] = m.nnod; out5[3] = m.ntri; out5[4] = (int32_t)m.nnz();
  if (x) std::copy(m.x.begin(), m.x.end(), x);
  if (y) std::copy(m.y.begin(), m.y.end(), y);
  if (z) std::copy(m.z.begin(), m.z.end(), z);
  if (tetra) std::copy(m.tetra.begin(), m.tetra.end(), tetra);
  if (rowptr) std::copy(m.rowptr.begin(), m.rowptr.end(), rowptr);
  if (cols) std::copy(m.cols.begin(), m.cols.end(), cols);
  return CATHY_GB300_OK;
}

int32_t cathy_gb300_create(int32_t nmembers, const cathy_member_t* members,
                           const cathy_opts_t* opts, void** handle) {
  if (!handle || nmembers <= 0 || !members) return CATHY_GB300_EINVAL;
  if (!have_device()) return CATHY_GB300_ENODEV;
  cathy_opts_t o = opts ? *opts : cathy_opts_t{0, 0, 0, 0.0, 0, 1};
  g_last_verbose = o.verbose;
  return guarded([&]() {
    *handle = engine_create(nmembers, members, o);
    return CATHY_GB300_OK;
  });
}

int32_t cathy_gb300_destroy(void* handle) {
  if (!handle) return CATHY_GB300_EINVAL;
  engine_destroy((Engine*)handle);
  return CATHY_GB300_OK;
}

int32_t cathy_gb300_sizes(void* h, int32_t m, int32_t* out5) {
  if (!h || !out5) return CATHY_GB300_EINVAL;
  return engine_sizes((Engine*)h, m, out5);
}

int32_t cathy_gb300_step(void* h, int32_t* nactive) {
  if (!h) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_step((Engine*)h, nactive); });
}

int32_t cathy_gb300_run(void* h, int32_t max_steps, int32_t* nsteps) {
  if (!h) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_run((Engine*)h, max_steps, nsteps); });
}

int32_t cathy_gb300_get_state(void* h, int32_t m, double* pnew, double* time,
                              double* deltat, int32_t* status) {
  if (!h) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_get_state((Engine*)h, m, pnew, time, deltat, status); });
}

int32_t cathy_gb300_get_saturation(void* h, int32_t m, double* sw) {
  if (!h || !sw) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_get_saturation((Engine*)h, m, sw); });
}

int32_t cathy_gb300_get_seepage(void* h, int32_t m, int32_t* sfex, double* sfq) {
  if (!h || !sfex || !sfq) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_get_seepage((Engine*)h, m, sfex, sfq); });
}

int32_t cathy_gb300_set_state(void* h, int32_t m, const double* ptimep, double time,
                              double deltat) {
  if (!h || !ptimep) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_set_state((Engine*)h, m, ptimep, time, deltat); });
}

int32_t cathy_gb300_num_records(void* h, int32_t m, int32_t* ni, int32_t* ns) {
  if (!h || !ni || !ns) return CATHY_GB300_EINVAL;
  return engine_num_records((Engine*)h, m, ni, ns);
}

int32_t cathy_gb300_get_records(void* h, int32_t m, cathy_iter_rec_t* ir,
                                cathy_step_rec_t* sr) {
  if (!h) return CATHY_GB300_EINVAL;
  return engine_get_records((Engine*)h, m, ir, sr);
}

int32_t cathy_gb300_get_mesh(void* h, int32_t m, double* x, double* y, double* z,
                             int32_t* tetra, int32_t* rowptr, int32_t* cols) {
  if (!h) return CATHY_GB300_EINVAL;
  return engine_get_mesh((Engine*)h, m, x, y, z, tetra, rowptr, cols);
}

int32_t cathy_gb300_picard_system(void* h, int32_t m, double* vals, double* rhs,
                                  double* xt5, int32_t* dirmask) {
  if (!h || !vals || !rhs || !xt5 || !dirmask) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_picard_system((Engine*)h, m, vals, rhs, xt5, dirmask); });
}

int32_t cathy_gb300_reset(void* h) {
  if (!h) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_reset((Engine*)h); });
}

int32_t cathy_gb300_profile(void* h, int32_t enable, double* spmv_ms,
                            int64_t* spmv_launches, double* spmv_bytes) {
  if (!h) return CATHY_GB300_EINVAL;
  return engine_profile((Engine*)h, enable, spmv_ms, spmv_launches, spmv_bytes);
}

int32_t cathy_gb300_autotune(void* h, int32_t nrep, int32_t* sched, double* ms) {
  if (!h || !sched || !ms) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_autotune((Engine*)h, nrep, sched, ms); });
}

int32_t cathy_gb300_set_schedule(void* h, int32_t asm_blocks, int32_t spmv_blocks,
                                 int32_t asm_staged, int32_t spmv_staged) {
  if (!h) return CATHY_GB300_EINVAL;
  return guarded([&]() {
    return engine_set_schedule((Engine*)h, asm_blocks, spmv_blocks, asm_staged, spmv_staged);
  });
}

int32_t cathy_gb300_phase_timers(void* h, int32_t enable, double* out, int32_t n) {
  if (!h || (n > 0 && !out) || n < 0) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_phase_timers((Engine*)h, enable, out, n); });
}

int32_t cathy_gb300_time_assembly(void* h, int32_t nrep, double* ms, double* bytes,
                                  int64_t* rows) {
  if (!h || !ms || !bytes || !rows) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_time_assembly((Engine*)h, nrep, ms, bytes, rows); });
}

int32_t cathy_gb300_stats(void* h, double* gpu_ms, int64_t* launches,
                          int64_t* lin_iters, int64_t* nl_iters) {
  if (!h) return CATHY_GB300_EINVAL;
  return engine_stats((Engine*)h, gpu_ms, launches, lin_iters, nl_iters);
}

int32_t cathy_gb300_attach_learned(void* h, void* model, int32_t mode) {
  if (!h || mode < 0 || mode > 2) return CATHY_GB300_EINVAL;
  return guarded([&]() { return engine_attach_learned((Engine*)h, model, mode); });
}

int32_t cathy_gb300_learned_stats(void* h, double* out, int32_t n) {
  if (!h || !out || n < 0) return CATHY_GB300_EINVAL;
  return engine_learned_stats((Engine*)h, out, n);
}

int32_t cathy_gb300_timers(void* h, double* out, int32_t n) {
  if (!h || !out || n < 0) return CATHY_GB300_EINVAL;
  return engine_timers((Engine*)h, out, n);
}

int32_t cathy_gb300_symslv(const int32_t* iout, const int32_t* n,
                           const int32_t* nterm, const int32_t* numdir,
                           int32_t* niter, const int32_t* itmxcg,
                           const double* tolcg, const double* rmin,
                           const int32_t* noddir, const int32_t* ja,
                           const int32_t* topol, double* pnew,
                           const double* tnoti, const double* coef1,
                           double* coef2, double* scr, double* err,
                           double* res) {
  (void)iout; (void)scr;
  if (!n || !nterm || !numdir || !niter || !itmxcg || !tolcg || !ja || !topol ||
      !pnew || !tnoti || !coef1 || *n <= 0 || *numdir < 0 || (*numdir > 0 && !noddir))
    return CATHY_GB300_EINVAL;
  if (!have_device()) return CATHY_GB300_ENODEV;
  return guarded([&]() {
    return dropin_symslv(*n, *nterm, *numdir, noddir, ja, topol, pnew, tnoti, coef1, coef2,
                         *itmxcg, *tolcg, rmin ? *rmin : 1.7e-100, niter, err, res);
  });
}

int32_t cathy_gb300_nsyslv(const int32_t* isolv, const int32_t* iout,
                           const int32_t* n, const int32_t* nterm,
                           const int32_t* numdir, const int32_t* noddir,
                           const int32_t* itmxcg, int32_t* niter,
                           const int32_t* ia, const int32_t* ja,
                           const int32_t* topol, const double* tolcg,
                           const double* rmin, const double* coef1,
                           double* coef2, double* pnew, const double* tnoti,
                           double* err, double* res) {
  (void)iout; (void)ia;
  if (!isolv || !n || !nterm || !numdir || !itmxcg || !niter || !ja || !topol ||
      !tolcg || !coef1 || !pnew || !tnoti || *n <= 0 || *numdir < 0 ||
      (*numdir > 0 && !noddir))
    return CATHY_GB300_EINVAL;
  if (!have_device()) return CATHY_GB300_ENODEV;
  return guarded([&]() {
    return dropin_nsyslv(*isolv, *n, *nterm, *numdir, noddir, ja, topol, pnew, tnoti, coef1,
                         coef2, *itmxcg, *tolcg, rmin ? *rmin : 1.7e-100, niter, err, res);
  });
}

int32_t cathy_gb300_asspic(const int32_t* nt, const int32_t* ntri,
                           const int32_t* tetra, const int32_t* tetja,
                           const double* lmass, double* coef1, double* coef2,
                           double* coef4, const double* et1e,
                           const double* pel, const double* permx,
                           const double* permy, const double* permz,
                           const double* ckrwe, const double* etae,
                           const double* volu, const double* volur,
                           const double* bi, const double* ci,
                           const double* di, const int32_t* maxstr,
                           const int32_t* nterm) {
  (void)etae;
  if (!nt || !ntri || !tetra || !tetja || !lmass || !coef1 || !coef2 || !coef4 ||
      !maxstr || !nterm || *nt <= 0)
    return CATHY_GB300_EINVAL;
  if (!have_device()) return CATHY_GB300_ENODEV;
  return guarded([&]() {
    return dropin_asspic(*nt, *ntri, tetra, tetja, lmass, coef1, coef2, coef4, et1e, pel,
                         permx, permy, permz, ckrwe, volur, volu, bi, ci, di, *maxstr, *nterm);
  });
}

}  // extern "C"
