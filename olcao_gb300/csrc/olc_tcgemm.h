// Blackwell tensor-core products of the mixed solver (olc_tcgemm.cu).
#pragma once

#include <cstdint>

#include "olc_common.h"

namespace olc {
namespace tc {

constexpr int kBeta = 8;         // bits per digit of the fixed-point split (|d| <= 255, exact in BF16)
constexpr int kMaxPairs = 96;    // digit pairs (or BF16-piece pairs) per launch

// One operand-plane pair of a launch; shift: int64 shift of its drained sums
// (fixed mode, negative = right shift).
struct TcPair {
  int8_t pa, pb;
  int16_t shift;
};

// Launch parameters (passed by value: no host memory is read at run time,
// so launches can be captured into a CUDA graph).
struct TcParams {
  int m, ncols, ldc;            // output rows, complex columns, leading dimension (complex elements)
  long long stride_c;           // batch stride of the output (complex elements)
  double* c64;                  // fixed mode output (complex FP64)
  float* c32;                   // f32 mode output (complex FP32)
  float alpha, beta;            // f32 mode: C = alpha D + beta C
  const int* ea;                // fixed mode: row exponents of op(A) [batch][m]
  const int* fb;                // fixed mode: column exponents of B [batch][ncols]
  int base;                     // fixed mode: output scale 2^(ea + fb + base)
  int planes_a, planes_b;       // planes per batch entry
  int nmt, nnt;                 // tiles
  int npairs, kblocks, chunk_blocks;   // segments: pairs x ceil(kblocks / chunk_blocks) K chunks
  int herm_upper;               // Hermitian result: tiles wholly below the diagonal are skipped
  int lower_only;               // f32 mode: tiles wholly above the diagonal are skipped
  int kp;                       // complex K per half of K' (K' = 2 kp)
  int tri_a_upper, tri_a_lower, tri_b_upper;   // triangular operands: zero K blocks skipped
  int* err;                     // device error word (expired waits)
  TcPair pairs[kMaxPairs];
};

// FP64-accurate complex product C[b] = op(A[b]) B[b] (m x n, column-major,
// ld m) from 8-bit digit planes: bits_a / bits_b bits kept of A / B.
// hermitian: the result is known to be Hermitian (m == n); only the tiles
// that touch the upper triangle are computed and the strict lower triangle
// is filled from it.
template <class TA, class TB>
int zgemm_fixed(olc_context* ctx, int m, int n, int k, const TA* A, long long sA, int lda, bool conjA, int bits_a,
                const TB* B, long long sB, int ldb, int bits_b, double* C, int nb, int stage,
                bool hermitian = false);

// Triangular operands of cgemm_f32: op(A) upper triangular (op(A)(r, k) = 0
// for k < r), op(A) lower triangular (zero for k > r), B upper triangular
// (B(k, c) = 0 for k > c).  Each output tile then skips the K blocks that
// meet only zeros.
constexpr int kTriAUpper = 1, kTriALower = 2, kTriBUpper = 4;

// FP32-accurate complex product C[b] = alpha op(A[b]) B[b] + beta C[b] from
// three BF16 pieces per FP32 operand (six piece pairs).  lower: only the
// output tiles that reach the lower triangle (row >= column) are formed; the
// rest of C keeps its values.  tri: kTri* flags of triangular operands.
int cgemm_f32(olc_context* ctx, int m, int n, int k, const float* A, long long sA, int lda, bool conjA,
              const float* B, long long sB, int ldb, float alpha, float beta, float* C, long long sC, int ldc,
              int nb, int stage, bool lower = false, int tri = 0);

// Digits and kept pairs of a fixed-point product (see olc_tcgemm.cu).
void fixed_plan(int bits_a, int bits_b, int prec, int* na, int* nbd, int* T);

// Reads and clears the device error word of the tensor-core kernels
// (non-zero: a pipeline wait expired).
int read_error(int* code);

}  // namespace tc
}  // namespace olc
