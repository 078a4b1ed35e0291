// Primitive kernels of the electronic-potential pass for the angular classes
// with an f function (l1 = 3 or l2 = 3), in all three precision modes,
// compiled in a translation unit of their own.
#include "olc_prim_kernel.cuh"

namespace olc {

int launch_prim_f_elecpot(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, int mode, dim3 g,
                          dim3 b) {
  switch ((l1 * 4 + l2) * 3 + mode) {
#define OLC_FCASE(L1, L2, M) \
  case (L1 * 4 + L2) * 3 + M: prim_kernel<OLC_OP_ELECPOT, L1, L2, M><<<g, b, 0, st>>>(v, a); break;
#define OLC_FCASES(L1, L2) OLC_FCASE(L1, L2, 0) OLC_FCASE(L1, L2, 1) OLC_FCASE(L1, L2, 2)
    OLC_FCASES(0, 3) OLC_FCASES(1, 3) OLC_FCASES(2, 3) OLC_FCASES(3, 0) OLC_FCASES(3, 1) OLC_FCASES(3, 2)
    OLC_FCASES(3, 3)
#undef OLC_FCASES
#undef OLC_FCASE
    default: return fail(OLC_ERR_ARG, "not an f class");
  }
  return cuda_check(cudaGetLastError(), "prim_kernel launch (f class)");
}

void launch_prim_batch_f_elecpot(int n, const double* in, const int32_t* lm, double* out) {
  launch_prim_batch_f_kind<4>(n, in, lm, out);
}

}  // namespace olc
