// The testing entry olc_primitive_batch for nuclear3CIntg with an f
// function, apart from the nuclear pass's kernels (each is large).
#include "olc_prim_kernel.cuh"

namespace olc {

void launch_prim_batch_f_nuclear(int n, const double* in, const int32_t* lm, double* out) {
  launch_prim_batch_f_kind<3>(n, in, lm, out);
}

}  // namespace olc
