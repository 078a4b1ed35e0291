// Internal declarations shared by the host set-up, the integral kernels and the
// dense linear-algebra stages of libolcao_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdint>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "olcao_gpu.h"

namespace olc {

constexpr double kPi = 3.141592653589793;
constexpr int kMaxL = 3;            // highest l the integral kernels are built for
constexpr int kMaxLm = 16;          // (kMaxL+1)^2 real harmonics s..f
constexpr int kNumClasses = (kMaxL + 1) * (kMaxL + 1);

// Per-atom-type data the kernels read (basis.f90:55-243 restated).
struct DevType {
  int32_t element;      // 0-based element id
  int32_t nalpha;       // numOrbAlphas(1)
  int32_t nstates;      // valence + core states
  int32_t nvale;
  int32_t ncore;
  int32_t lmax_alpha[OLC_MAX_ALPHAS];   // l range available at each exponent
  int32_t lm_index[OLC_MAX_STATES];     // 1-based lm of each state
  double alphas[OLC_MAX_ALPHAS];
  double basis[OLC_MAX_ALPHAS * OLC_MAX_STATES];   // [alpha][state]
};

// One surviving atom pair (i <= j) with its nearest-image lattice vector.
struct DevPair {
  int32_t i, j;
  int32_t task_begin, task_end;   // its (pair, cell) tasks
  double L[3];
};

// One (pair, cell) block.
struct DevTask {
  int32_t pair;
  int32_t cell;
  double sep;                    // |A - B - L - R|^2
};

// Potential sites grouped by type (potSites, potTypes).
struct DevPotType {
  int32_t element;
  int32_t num_alphas;
  int32_t first_site;
  int32_t multiplicity;
  int32_t cumul_alpha;
  double nuc_charge;
  double nuc_alpha;
  double alphas[OLC_MAX_POT_ALPHAS];
};

// Everything a kernel needs about the system, passed by value.
struct SysView {
  const DevType* types;
  const int32_t* site_type;
  const double* site_pos;            // [3*n]
  const int32_t* cum_vale;
  const int32_t* cum_core;
  const DevPair* pairs;
  const DevTask* tasks;
  const double* cells;               // [4*ncells] (x, y, z, |R|^2) sorted
  int32_t ncells;
  const DevPotType* pot_types;
  int32_t num_pot_types;
  const double* pot_site_pos;        // [3*npotsites]
  const int32_t* pot_site_type;
  int32_t num_pot_sites;
  const double* elem_alpha;          // [nelem*OLC_MAX_ALPHAS]
  const double* elem_nuc_alpha;      // [nelem]
  const double* elem_pot_alpha;      // [nelem*OLC_MAX_POT_ALPHAS]
  double inv_real[9];                // invRealVectors(i, xyz) row-major [abc][xyz]
  double real_vec[9];                // [abc][xyz]
  double log_thresh;                 // T = -ln(BASIS_FN thresh)
  int32_t vale_dim, core_dim, nk;
  const double* kxyz;                // [3*nk]
  const double* phase;               // [nk*ncells] complex (re,im) : exp(i k.R)
};

// Items of the primitive stage: one per (task, alpha1, alpha2) grouped by
// (l1, l2) class; within a class ordered by task.
struct ItemLists {
  int32_t count[kNumClasses];
  int64_t sh_offset[kNumClasses];       // offset (doubles) of the class block in scratch
  int32_t* task[kNumClasses];           // device arrays
  int32_t* ab[kNumClasses];             // alpha1 | alpha2 << 8
  int32_t* task_start[kNumClasses];     // [ntasks+1] start of each task's items
  int64_t total_sh;                     // doubles of sh scratch
};

// Per-stage CUDA-event timing on the context stream.
struct StageEvent {
  int stage;
  cudaEvent_t a, b;
};

}  // namespace olc

struct olc_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaMemPool_t pool = nullptr;        // scratch of the SCF pass, kept between calls
  // CUDA graph of the mixed stored-form pass (OLC_ITER_GRAPH)
  cudaGraphExec_t graph_exec = nullptr;
  int graph_key = -1, graph_warm = -1;
  bool graph_broken = false, capturing = false;
  int64_t graph_launches = 0;
  double* g_coeff = nullptr;
  double* g_eig = nullptr;
  double* g_vec = nullptr;
  // FP32 inverse Cholesky factors U^{-1} of the prepared S(k) (they do not
  // change between SCF passes; FP64 factorisation): [nk][n][n], valid after
  // the first mixed pass
  float* w32 = nullptr;
  bool w32_valid = false;
  // tuned CTAs per k of the FP32 tridiagonalisation (olc_tridiag.cu)
  int trd_tuned_n = 0, trd_tuned_nk = 0, trd_tuned_g = 0;
  cusolverDnHandle_t solver = nullptr;
  // host copies
  olc_dims_t dims{};
  int nelem = 0;
  std::vector<olc::DevType> htypes;
  std::vector<olc::DevPotType> hpots;
  std::vector<olc::DevPair> hpairs;
  std::vector<olc::DevTask> htasks;
  std::vector<double> hcells;
  // device
  olc::SysView view{};
  std::vector<void*> allocations;
  olc::ItemLists items{};
  double* d_sh = nullptr;          // primitive sh scratch
  double* d_block = nullptr;       // contracted (task, m1, m2) blocks
  int64_t block_stride = 0;        // doubles per task block (MS*MS)
  int max_states = 0;
  // cached iteration-invariant data (olc_scf_prepare)
  int rel = 0;                     // 1: mass-velocity term in H (scalar relativistic)
  bool prepared = false;
  int prep_precision = 0;
  int prep_form = 0;
  double* d_terms = nullptr;       // stored form: packed NP, KE, (MV), V_j [2+rel+pd][nk][plen][2]
  double* d_scv = nullptr;         // S core-vale  [nk][nv][nc] complex
  double* d_h0 = nullptr;          // ortho(KE + NP) full upper [nk][nv][nv] complex
  double* d_chol = nullptr;        // Cholesky factor of ortho'd S, [nk][nv][nv]
  double* d_work_vv = nullptr;
  double* d_work_cv = nullptr;
  double* d_work_cc = nullptr;
  double* d_work_x = nullptr;      // GEMM temporaries
  double* d_work_y = nullptr;
  double* d_work_w = nullptr;
  void* d_solver_work = nullptr;
  size_t solver_work_bytes = 0;
  // independent k-point solves run concurrently on sub-streams
  std::vector<cudaStream_t> sub_streams;
  std::vector<cusolverDnHandle_t> sub_solvers;
  std::vector<void*> sub_work;
  std::vector<double*> sub_eval;
  size_t sub_work_bytes = 0;
  int sub_n = 0;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_join;
  // FP32 solves of the mixed-precision path
  std::vector<cudaStream_t> mixed_streams;
  std::vector<cusolverDnHandle_t> mixed_solvers;
  std::vector<void*> mixed_work;
  std::vector<cudaEvent_t> mixed_join;
  int mixed_n = 0;
  int mixed_lwork = 0;
  int* d_info = nullptr;
  bool info_potrf = false;         // d_info holds potrf's info (else chegvd's)
  double* d_eval = nullptr;
  // profiling
  bool profiling = false;
  std::vector<olc::StageEvent> prof_pending;
  std::vector<cudaEvent_t> prof_pool;
  double prof_ms[OLC_NUM_STAGES] = {};
  int64_t prof_launches[OLC_NUM_STAGES] = {};
  double prof_flops[OLC_NUM_STAGES] = {};
  double prof_bytes[OLC_NUM_STAGES] = {};
};

namespace olc {

// Stream-ordered scratch from the context's own pool: the pool keeps freed
// memory (release threshold = max), so repeated SCF passes do not go back to
// the CUDA driver for their tens of GB of scratch.
inline cudaError_t ctx_malloc(olc_context* ctx, void** p, size_t bytes, cudaStream_t s) {
  return ctx->pool ? cudaMallocFromPoolAsync(p, bytes, ctx->pool, s) : cudaMallocAsync(p, bytes, s);
}

void set_error(const std::string& msg);
void count_launch(int n = 1);
// Algorithmic work of a stage (tensor flops or streamed bytes), counted
// while the context is profiling.
inline void add_work(olc_context* ctx, int stage, double flops, double bytes) {
  if (!ctx || !ctx->profiling || ctx->capturing) return;
  ctx->prof_flops[stage] += flops;
  ctx->prof_bytes[stage] += bytes;
}

// Records a stage's start on construction and its end on destruction when the
// context is profiling; `launches` kernels are attributed to the stage.
class StageScope {
 public:
  StageScope(olc_context* ctx, int stage, int launches = 1);
  ~StageScope();
  void add_launches(int n);
 private:
  olc_context* ctx_;
  int stage_;
  int launches_;
  cudaEvent_t a_ = nullptr;
};
int fail(int code, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

// device allocation tracked by the context
template <class T>
int dalloc(olc_context* ctx, T** p, size_t count) {
  void* q = nullptr;
  if (count == 0) { *p = nullptr; return OLC_OK; }
  cudaError_t e = cudaMalloc(&q, count * sizeof(T));
  if (e != cudaSuccess) return fail(OLC_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  ctx->allocations.push_back(q);
  *p = static_cast<T*>(q);
  return OLC_OK;
}

// Runs fn(i) for i in [0, nthreads) on separate host threads with `device`
// current.  Library calls that block their host thread (cuSOLVER's divide and
// conquer waits on the device) overlap only when issued from different
// threads.  Returns the first non-zero status.
inline int parallel_host(int nthreads, int device, const std::function<int(int)>& fn) {
  std::vector<int> status(nthreads, 0);
  std::vector<std::thread> pool;
  pool.reserve(nthreads);
  for (int i = 0; i < nthreads; ++i)
    pool.emplace_back([&, i]() {
      cudaSetDevice(device);
      status[i] = fn(i);
    });
  for (auto& t : pool) t.join();
  for (int v : status)
    if (v) return v;
  return 0;
}

// host set-up (olc_setup.cpp)
int build_system(olc_context* ctx, const olc_system_t* sys);

// integral stages (olc_integrals.cu)
int run_primitives(olc_context* ctx, int op, int term, const double* coeffs,
                   int precision, bool accumulate);
int run_contract_bloch(olc_context* ctx, double* vv, double* cv, double* cc);
int primitive_batch_device(int kind, int n, const double* in, const int32_t* lmalpha,
                           double* out);

// dense stages (olc_linalg.cu)
int ortho_pack(olc_context* ctx, bool is_overlap, double* vv, const double* cv,
               const double* cc, const double* scv, double* packed, double* full_out);
int assemble_packed(olc_context* ctx, const double* const* terms, const double* coeffs,
                    int nterm, double* out);
int solve_packed(olc_context* ctx, const double* packed_h, const double* packed_s,
                 int num_states, double* eigenvalues, double* vectors, int32_t* info);
int scf_prepare(olc_context* ctx, int precision, int form);
int scf_matrices(olc_context* ctx, const double* coeffs, int kpoint, double* h, double* s,
                 int on_device);
int scf_iteration(olc_context* ctx, const double* coeffs, int precision, int num_states,
                  double* eigenvalues, int flags, double* vectors);

// FP64-accurate complex products from BF16 tensor-core digits (olc_ozaki.cu,
// on the tcgen05 kernel of olc_tcgemm.cu):
// C[b] = op(A[b]) B[b], A logical m x k (conjA: A = src^H), B k x n, C m x n
// complex FP64 with batch stride m*n; bits_a/bits_b = bits kept per operand;
// batch strides sA, sB count elements of TA / TB (two per complex number).
// hermitian: the product is known to be Hermitian (only its upper part is
// formed, the lower filled by symmetry).
template <class TA, class TB>
int ozaki_zgemm(olc_context* ctx, int m, int n, int k, const TA* A, long long sA, int lda,
                bool conjA, int bits_a, const TB* B, long long sB, int ldb, int bits_b, double* C,
                int nb, int stage = OLC_STAGE_REFINE, bool hermitian = false);

// status of a queued mixed solve (olc_mixed.cu)
int mixed_check_info(olc_context* ctx);

// occupations (olc_populate.cpp, host)
int populate_states(int num_states, int nk, int spin, const double* eig, const double* kweight,
                    double num_electrons, double thermal_sigma, double fermi_search_limit,
                    double max_thermal_range, double* occupation, double* occupied_energy);

// valence density and its traces (olc_density.cu)
int make_valence_rho(olc_context* ctx, int num_states, int spin, const double* occupation,
                     const double* eigenvalues, const double* vectors, double* traces,
                     double* electron_energy, double* rho_packed);

// raw layout-identical dataset writer (olc_layout.cu)
int write_setup_integrals(olc_context* ctx, const char* root);
int write_eigen(const char* root, int nk, int spin, int num_states, int vale_dim, const double* eig,
                const double* vectors);

// batched FP32 eigen-solve (olc_tridiag.cu)
int hetrd_max_n();
int inverse_factors(olc_context* ctx, int n, int nk, const double* s64, float* w32);
int solve_fp32_batched(olc_context* ctx, int n, int nk, const float* h32, const float* w32, float* X);

}  // namespace olc
