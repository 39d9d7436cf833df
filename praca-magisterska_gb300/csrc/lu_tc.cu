// lu_tc.cu -- FP32 trailing-update GEMM of the precision-form LU on the tensor
// cores (tcgen05).  Placeholder: the SIMT GEMM is used until this path lands.
#include "solve_internal.h"

namespace wmom {
GemmHook<float2> tc_gemm_hook() { return nullptr; }
}  // namespace wmom
