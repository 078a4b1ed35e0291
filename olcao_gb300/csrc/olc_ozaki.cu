// FP64-accurate complex products C[b] = op(A[b]) B[b] (the error-free
// splitting of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012)
// 95-118): every row of op(A) and column of B is scaled by a power of two and
// cut into signed digits that BF16 holds exactly, the digit products run on
// the hand-written tcgen05 kernel of olc_tcgemm.cu (fixed mode), which sums
// them in 64-bit fixed point in its epilogue.  This file is the entry the
// solver, the orthogonalisation and the density step call.
#include "olc_common.h"
#include "olc_tcgemm.h"

namespace olc {

template <class TA, class TB>
int ozaki_zgemm(olc_context* ctx, int m, int n, int k, const TA* A, long long sA, int lda,
                bool conjA, int bits_a, const TB* B, long long sB, int ldb, int bits_b, double* C,
                int nb, int stage, bool hermitian) {
  return tc::zgemm_fixed<TA, TB>(ctx, m, n, k, A, sA, lda, conjA, bits_a, B, sB, ldb, bits_b, C, nb, stage,
                                 hermitian);
}

template int ozaki_zgemm<double, float>(olc_context*, int, int, int, const double*, long long, int, bool,
                                        int, const float*, long long, int, int, double*, int, int, bool);
template int ozaki_zgemm<float, double>(olc_context*, int, int, int, const float*, long long, int, bool,
                                        int, const double*, long long, int, int, double*, int, int, bool);
template int ozaki_zgemm<double, double>(olc_context*, int, int, int, const double*, long long, int, bool,
                                         int, const double*, long long, int, int, double*, int, int, bool);

}  // namespace olc
