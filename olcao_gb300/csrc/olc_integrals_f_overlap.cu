// Primitive kernels of the overlap pass for the angular classes with an f
// function (l1 = 3 or l2 = 3), compiled in a translation unit of their own.
#include "olc_prim_kernel.cuh"

namespace olc {

int launch_prim_f_overlap(cudaStream_t st, const SysView& v, const PrimArgs& a, int l1, int l2, dim3 g, dim3 b) {
  switch (l1 * 4 + l2) {
#define OLC_FCASE(L1, L2) \
  case L1 * 4 + L2: prim_kernel<OLC_OP_OVERLAP, L1, L2, 0><<<g, b, 0, st>>>(v, a); break;
    OLC_FCASE(0, 3) OLC_FCASE(1, 3) OLC_FCASE(2, 3) OLC_FCASE(3, 0) OLC_FCASE(3, 1) OLC_FCASE(3, 2) OLC_FCASE(3, 3)
#undef OLC_FCASE
    default: return fail(OLC_ERR_ARG, "not an f class");
  }
  return cuda_check(cudaGetLastError(), "prim_kernel launch (f class)");
}

void launch_prim_batch_f_overlap(int n, const double* in, const int32_t* lm, double* out) {
  launch_prim_batch_f_kind<1>(n, in, lm, out);
}

void launch_prim_batch_f_momentum(int kind, int n, const double* in, const int32_t* lm, double* out) {
  if (kind == 6) launch_prim_batch_f_kind<6>(n, in, lm, out);
  else if (kind == 7) launch_prim_batch_f_kind<7>(n, in, lm, out);
  else launch_prim_batch_f_kind<8>(n, in, lm, out);
}

}  // namespace olc
