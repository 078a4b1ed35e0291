// Allocation-free entry point: the batched small-n generalised eigen-solve
// from packed H(k), S(k), with its unpacked working copies held in a
// file-scope device array instead of memory obtained from cudaMalloc.
//
// Who needs it: callers that may not allocate device memory once their SCF
// loop is running -- a host program (a Fortran driver, say) that reserves all
// device memory for its own pool at start-up and forbids allocation inside the
// loop, or a framework that owns the device allocator and does not let
// libraries call cudaMalloc/cudaFree.  They pass device pointers for every
// input and output; this call allocates nothing.
#include <mutex>
#include <string>

#include "olc_common.h"

namespace olc {

int launch_small_hegv_raw(cudaStream_t stream, const double* h_full, const double* s_full, int n,
                          int nk, int num_states, double* eigenvalues, double* vectors,
                          int32_t* info_dev);
int small_solver_capacity_n();

namespace {

// 16 MiB of working space on every device that loads the library, held until
// the process exits: the unpacked H and S of all k-points,
// 2 matrices x nk x n x n complex128 <= kScratchDoubles doubles.
constexpr size_t kScratchDoubles = (size_t)2 * 1024 * 1024;
__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Host-side addresses of g_noalloc_scratch per device (the symbol's name in
// host code is only a stand-in; the device address comes from
// cudaGetSymbolAddress with the device current).
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(double** out) {
  int dev = 0;
  int st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (st) return st;
  if (dev < 0 || dev >= kMaxDevices) return fail(OLC_ERR_ARG, "device index beyond the supported range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    st = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
    if (st) return st;
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return OLC_OK;
}

// packed [nk][n(n+1)/2][2] -> full Hermitian [nk][n][n] (column-major)
__global__ void unpack_into_scratch(const double* __restrict__ packed, double* __restrict__ full,
                                    int n, int nk) {
  const size_t nn = (size_t)n * n;
  const size_t total = nn * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / nn);
    const size_t r = idx % nn;
    const int col = (int)(r / n), row = (int)(r % n);
    const int i = max(row, col), j = min(row, col);
    const size_t p = (size_t)k * ((size_t)n * (n + 1) / 2) + (size_t)i * (i + 1) / 2 + j;
    double re = packed[2 * p], im = packed[2 * p + 1];
    if (row > col) im = -im;
    if (row == col) im = 0.0;
    full[2 * idx] = re;
    full[2 * idx + 1] = im;
  }
}

}  // namespace
}  // namespace olc

using namespace olc;

extern "C" int olc_solve_zhegv_noalloc(int n, int nk, const double* packed_h,
                                       const double* packed_s, int num_states,
                                       double* eigenvalues, double* vectors, int32_t* info,
                                       void* stream) {
  if (n < 1 || nk < 1 || !packed_h || !packed_s || !eigenvalues || !info)
    return fail(OLC_ERR_ARG, "olc_solve_zhegv_noalloc: null or empty argument");
  if (num_states < 1 || num_states > n)
    return fail(OLC_ERR_ARG, "olc_solve_zhegv_noalloc: num_states out of range");
  const int nmax = small_solver_capacity_n();
  if (n > nmax)
    return fail(OLC_ERR_ARG, "olc_solve_zhegv_noalloc: n exceeds " + std::to_string(nmax) +
                                 ", the largest size this allocation-free solver handles");
  const size_t need = (size_t)4 * n * n * nk;   // H and S, complex128
  if (need > kScratchDoubles)
    return fail(OLC_ERR_ARG, "olc_solve_zhegv_noalloc: nk * n * n exceeds " +
                                 std::to_string(kScratchDoubles / 4) + ", the capacity of its " +
                                 std::to_string(kScratchDoubles * 8 >> 20) +
                                 " MiB working array; split the k-points into batches");
  double* scratch = nullptr;
  int st = scratch_for_current_device(&scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* h = scratch;
  double* sm = scratch + (size_t)2 * n * n * nk;
  const size_t total = (size_t)n * n * nk;
  const int grid = (int)std::min<size_t>((total + 255) / 256, 152 * 32);
  count_launch(2);
  unpack_into_scratch<<<grid, 256, 0, s>>>(packed_h, h, n, nk);
  unpack_into_scratch<<<grid, 256, 0, s>>>(packed_s, sm, n, nk);
  if ((st = cuda_check(cudaGetLastError(), "unpack_into_scratch"))) return st;
  return launch_small_hegv_raw(s, h, sm, n, nk, num_states, eigenvalues, vectors, info);
}
