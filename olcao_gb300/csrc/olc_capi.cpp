// C ABI of libolcao_gb300 (declared in include/olcao_gpu.h).
#include <cstdlib>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "olc_common.h"
#include "olc_tcgemm.h"

namespace olc {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

namespace {
std::atomic<int64_t> g_launches{0};

cudaEvent_t take_event(olc_context* ctx) {
  if (!ctx->prof_pool.empty()) {
    cudaEvent_t e = ctx->prof_pool.back();
    ctx->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void drain_profile(olc_context* ctx) {
  cudaStreamSynchronize(ctx->stream);
  for (auto& r : ctx->prof_pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) ctx->prof_ms[r.stage] += ms;
    ctx->prof_pool.push_back(r.a);
    ctx->prof_pool.push_back(r.b);
  }
  ctx->prof_pending.clear();
}
}  // namespace

void count_launch(int n) { g_launches += n; }

StageScope::StageScope(olc_context* ctx, int stage, int launches)
    : ctx_(ctx), stage_(stage), launches_(launches) {
  count_launch(launches);
  if (ctx_ && ctx_->profiling && !ctx_->capturing) {
    a_ = take_event(ctx_);
    cudaEventRecord(a_, ctx_->stream);
  }
}

void StageScope::add_launches(int n) {
  launches_ += n;
  count_launch(n);
}

StageScope::~StageScope() {
  if (!ctx_) return;
  if (ctx_->profiling && a_) {
    cudaEvent_t b = take_event(ctx_);
    cudaEventRecord(b, ctx_->stream);
    ctx_->prof_pending.push_back(StageEvent{stage_, a_, b});
  }
  ctx_->prof_launches[stage_] += launches_;
}

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return OLC_OK;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? OLC_ERR_ALLOC : OLC_ERR_CUDA;
}

int build_phase_table(olc_context* ctx);
int ozaki_selftest(olc_context* ctx, int m, int n, int k, const double* A, const double* B,
                   double* C);
int ortho_pack_ex(olc_context* ctx, bool is_overlap, const double* vv, const double* cv,
                  const double* cc, const double* scv, double* packed, double* full,
                  const double* add);

}  // namespace olc

using namespace olc;

extern "C" {

const char* olc_version(void) { return "olcao_gb300 0.1 (sm_103a)"; }

int olc_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return OLC_ERR_ARG;
  std::snprintf(buf, len, "%s", g_last_error.c_str());
  return OLC_OK;
}

int olc_create(const olc_system_t* sys, void* stream, olc_context_t** out) {
  if (!out) return fail(OLC_ERR_ARG, "olc_create: null output");
  *out = nullptr;
  if (!sys) return fail(OLC_ERR_ARG, "olc_create: null system");
  int dev = 0;
  int st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (st) return st;
  olc_context* ctx = new olc_context();
  ctx->device = dev;
  ctx->stream = static_cast<cudaStream_t>(stream);
  if (cusolverDnCreate(&ctx->solver) != CUSOLVER_STATUS_SUCCESS) {
    delete ctx;
    return fail(OLC_ERR_CUDA, "cusolverDnCreate failed");
  }
  cusolverDnSetStream(ctx->solver, ctx->stream);
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess) {
      ctx->pool = nullptr;
      olc_destroy(ctx);
      return fail(OLC_ERR_CUDA, "cudaMemPoolCreate failed");
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  st = build_system(ctx, sys);
  if (!st) st = build_phase_table(ctx);
  if (!st) st = cuda_check(cudaStreamSynchronize(ctx->stream), "olc_create sync");
  if (st) {
    std::string keep = g_last_error;
    olc_destroy(ctx);
    g_last_error = keep;
    return st;
  }
  *out = ctx;
  return OLC_OK;
}

int olc_destroy(olc_context_t* ctx) {
  if (!ctx) return OLC_OK;
  cudaStreamSynchronize(ctx->stream);
  drain_profile(ctx);
  for (cudaEvent_t e : ctx->prof_pool) cudaEventDestroy(e);
  for (void* p : ctx->allocations) cudaFree(p);
  if (ctx->d_solver_work) cudaFree(ctx->d_solver_work);
  for (size_t i = 0; i < ctx->sub_streams.size(); ++i) {
    cudaStreamSynchronize(ctx->sub_streams[i]);
    cusolverDnDestroy(ctx->sub_solvers[i]);
    cudaFree(ctx->sub_work[i]);
    cudaFree(ctx->sub_eval[i]);
    cudaStreamDestroy(ctx->sub_streams[i]);
    cudaEventDestroy(ctx->ev_join[i]);
  }
  for (size_t i = 0; i < ctx->mixed_streams.size(); ++i) {
    cudaStreamSynchronize(ctx->mixed_streams[i]);
    cusolverDnDestroy(ctx->mixed_solvers[i]);
    cudaFree(ctx->mixed_work[i]);
    cudaStreamDestroy(ctx->mixed_streams[i]);
    cudaEventDestroy(ctx->mixed_join[i]);
  }
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->pool) {
    cudaStreamSynchronize(ctx->stream);
    cudaMemPoolDestroy(ctx->pool);
  }
  if (ctx->solver) cusolverDnDestroy(ctx->solver);
  delete ctx;
  return OLC_OK;
}

int olc_get_dims(const olc_context_t* ctx, olc_dims_t* dims) {
  if (!ctx || !dims) return fail(OLC_ERR_ARG, "olc_get_dims: null argument");
  *dims = ctx->dims;
  return OLC_OK;
}

int olc_set_stream(olc_context_t* ctx, void* stream) {
  if (!ctx) return fail(OLC_ERR_ARG, "olc_set_stream: null context");
  ctx->stream = static_cast<cudaStream_t>(stream);
  cusolverDnSetStream(ctx->solver, ctx->stream);
  return OLC_OK;
}

int olc_gauss_overlap(olc_context_t* ctx, int op, int term, const double* coeffs, int precision,
                      double* vv, double* cv, double* cc) {
  if (!ctx || !vv) return fail(OLC_ERR_ARG, "olc_gauss_overlap: null argument");
  int st;
  if (op == OLC_OP_HAMILTONIAN) {
    if (!coeffs) return fail(OLC_ERR_ARG, "OLC_OP_HAMILTONIAN needs coefficients");
    const int pd = ctx->dims.pot_dim;
    std::vector<double> c(coeffs, coeffs + pd);
    double* dco = nullptr;
    if ((st = cuda_check(ctx_malloc(ctx, (void**)&dco, sizeof(double) * std::max(1, pd), ctx->stream), "malloc"))) return st;
    cudaMemcpyAsync(dco, c.data(), sizeof(double) * pd, cudaMemcpyHostToDevice, ctx->stream);
    st = run_primitives(ctx, OLC_OP_KINETIC, 0, nullptr, precision, false);
    if (!st) st = run_primitives(ctx, OLC_OP_NUCLEAR, 0, nullptr, precision, true);
    if (!st && ctx->rel) st = run_primitives(ctx, OLC_OP_MASSVEL, 0, nullptr, precision, true);
    if (!st) st = run_primitives(ctx, OLC_OP_ELECPOT, 0, dco, precision, true);
    cudaFreeAsync(dco, ctx->stream);
  } else if (op >= OLC_OP_OVERLAP && op <= OLC_OP_MASSVEL) {
    if (op == OLC_OP_ELECPOT && (term < 0 || term >= ctx->dims.pot_dim))
      return fail(OLC_ERR_ARG, "potential term out of range");
    st = run_primitives(ctx, op, term, nullptr, precision, false);
  } else {
    return fail(OLC_ERR_ARG, "unknown operator");
  }
  if (st) return st;
  st = run_contract_bloch(ctx, vv, cv, cc);
  if (st) return st;
  return cuda_check(cudaStreamSynchronize(ctx->stream), "olc_gauss_overlap sync");
}

int olc_ortho_pack(olc_context_t* ctx, int is_overlap, double* vv, const double* cv,
                   const double* cc, const double* s_cv, double* packed) {
  if (!ctx || !vv || !packed) return fail(OLC_ERR_ARG, "olc_ortho_pack: null argument");
  if (ctx->dims.core_dim && (!cv || !cc || !s_cv))
    return fail(OLC_ERR_ARG, "olc_ortho_pack: core blocks required");
  int st = ortho_pack_ex(ctx, is_overlap != 0, vv, cv, cc, is_overlap ? cv : s_cv, packed,
                         nullptr, nullptr);
  if (st) return st;
  return cuda_check(cudaStreamSynchronize(ctx->stream), "olc_ortho_pack sync");
}

int olc_assemble_hamiltonian(olc_context_t* ctx, const double* const* terms, const double* coeffs,
                             int nterm, double* packed_h) {
  if (!ctx || !terms || !coeffs || !packed_h) return fail(OLC_ERR_ARG, "olc_assemble_hamiltonian: null argument");
  return assemble_packed(ctx, terms, coeffs, nterm, packed_h);
}

int olc_solve_zhegv(olc_context_t* ctx, const double* packed_h, const double* packed_s,
                    int num_states, double* eigenvalues, double* vectors, int32_t* info) {
  if (!ctx || !packed_h || !packed_s || !eigenvalues) return fail(OLC_ERR_ARG, "olc_solve_zhegv: null argument");
  return solve_packed(ctx, packed_h, packed_s, num_states, eigenvalues, vectors, info);
}

int olc_scf_prepare(olc_context_t* ctx, int precision, int form) {
  if (!ctx) return fail(OLC_ERR_ARG, "olc_scf_prepare: null context");
  if (form != OLC_FORM_FUSED && form != OLC_FORM_STORED) return fail(OLC_ERR_ARG, "olc_scf_prepare: bad form");
  return scf_prepare(ctx, precision, form);
}

int olc_scf_iteration(olc_context_t* ctx, const double* coeffs, int precision, int num_states,
                      double* eigenvalues, int flags, double* vectors) {
  if (!ctx || !coeffs || !eigenvalues) return fail(OLC_ERR_ARG, "olc_scf_iteration: null argument");
  return scf_iteration(ctx, coeffs, precision, num_states, eigenvalues, flags, vectors);
}

int olc_scf_matrices(olc_context_t* ctx, const double* coeffs, int kpoint, double* h, double* s,
                     int on_device) {
  if (!ctx || !coeffs) return fail(OLC_ERR_ARG, "olc_scf_matrices: null argument");
  return scf_matrices(ctx, coeffs, kpoint, h, s, on_device);
}

int olc_split_zgemm(olc_context_t* ctx, int m, int n, int k, const double* a, const double* b,
                    double* c) {
  if (!ctx || !a || !b || !c || m < 1 || n < 1 || k < 1)
    return fail(OLC_ERR_ARG, "olc_split_zgemm: bad argument");
  return ozaki_selftest(ctx, m, n, k, a, b, c);
}

int olc_split_cgemm32(olc_context_t* ctx, int m, int n, int k, const float* a, int conj_a, const float* b,
                      float* c) {
  if (!ctx || !a || !b || !c || m < 1 || n < 1 || k < 1)
    return fail(OLC_ERR_ARG, "olc_split_cgemm32: bad argument");
  int st = tc::cgemm_f32(ctx, m, n, k, a, 0, conj_a ? k : m, conj_a != 0, b, 0, k, 1.0f, 0.0f, c, 0, m, 1,
                         OLC_STAGE_REFINE);
  int s2 = cuda_check(cudaStreamSynchronize(ctx->stream), "olc_split_cgemm32 sync");
  if (st || s2) return st ? st : s2;
  int code = 0;
  if ((st = tc::read_error(&code))) return st;
  if (code) return fail(OLC_ERR_CUDA, "tensor-core product: a pipeline wait expired");
  return OLC_OK;
}

int olc_profile_enable(olc_context_t* ctx, int on) {
  if (!ctx) return fail(OLC_ERR_ARG, "olc_profile_enable: null context");
  ctx->profiling = on != 0;
  return OLC_OK;
}

int olc_profile_reset(olc_context_t* ctx) {
  if (!ctx) return fail(OLC_ERR_ARG, "olc_profile_reset: null context");
  drain_profile(ctx);
  for (int s = 0; s < OLC_NUM_STAGES; ++s) {
    ctx->prof_ms[s] = 0.0;
    ctx->prof_launches[s] = 0;
    ctx->prof_flops[s] = 0.0;
    ctx->prof_bytes[s] = 0.0;
  }
  return OLC_OK;
}

int olc_profile_read(olc_context_t* ctx, int stage, int64_t* launches, double* ms) {
  if (!ctx || stage < 0 || stage >= OLC_NUM_STAGES) return fail(OLC_ERR_ARG, "olc_profile_read: bad argument");
  drain_profile(ctx);
  if (launches) *launches = ctx->prof_launches[stage];
  if (ms) *ms = ctx->prof_ms[stage];
  return OLC_OK;
}

int olc_profile_read_work(olc_context_t* ctx, int stage, double* flops, double* bytes) {
  if (!ctx || stage < 0 || stage >= OLC_NUM_STAGES)
    return fail(OLC_ERR_ARG, "olc_profile_read_work: bad argument");
  if (flops) *flops = ctx->prof_flops[stage];
  if (bytes) *bytes = ctx->prof_bytes[stage];
  return OLC_OK;
}

int64_t olc_launch_count(void) { return g_launches.load(); }

int olc_primitive_batch(int kind, int n, const double* in, const int32_t* lmalpha, double* out) {
  if (n > 0 && (!in || !lmalpha || !out)) return fail(OLC_ERR_ARG, "olc_primitive_batch: null argument");
  return primitive_batch_device(kind, n, in, lmalpha, out);
}

int olc_write_setup_integrals(olc_context_t* ctx, const char* root) {
  if (!ctx || !root) return fail(OLC_ERR_ARG, "olc_write_setup_integrals: null argument");
  return write_setup_integrals(ctx, root);
}

int olc_write_eigen(const char* root, int num_kpoints, int spin, int num_states, int vale_dim,
                    const double* eigenvalues, const double* vectors) {
  if (!root || !eigenvalues || num_kpoints < 1 || spin < 1 || num_states < 1 || vale_dim < 1 ||
      num_states > vale_dim)
    return fail(OLC_ERR_ARG, "olc_write_eigen: bad argument");
  return write_eigen(root, num_kpoints, spin, num_states, vale_dim, eigenvalues, vectors);
}

int olc_populate_states(int num_states, int num_kpoints, int spin, const double* eigenvalues,
                        const double* kpoint_weights, double num_electrons, double thermal_sigma,
                        double fermi_search_limit, double max_thermal_range, double* occupation,
                        double* occupied_energy) {
  if (num_states < 1 || num_kpoints < 1 || (spin != 1 && spin != 2) || !eigenvalues || !kpoint_weights ||
      !occupation || !(num_electrons >= 0.0) || !(thermal_sigma >= 0.0) ||
      (thermal_sigma > 0.0 && !(max_thermal_range > 0.0)))
    return fail(OLC_ERR_ARG, "olc_populate_states: bad argument");
  return populate_states(num_states, num_kpoints, spin, eigenvalues, kpoint_weights, num_electrons,
                         thermal_sigma, fermi_search_limit, max_thermal_range, occupation, occupied_energy);
}

int olc_make_valence_rho(olc_context_t* ctx, int num_states, int spin, const double* occupation,
                         const double* eigenvalues, const double* vectors, double* traces,
                         double* electron_energy, double* rho_packed) {
  if (!ctx) return fail(OLC_ERR_ARG, "olc_make_valence_rho: null context");
  return make_valence_rho(ctx, num_states, spin, occupation, eigenvalues, vectors, traces, electron_energy,
                          rho_packed);
}

}  // extern "C"
