// Tensor-core (tcgen05) paths: Gram matrices and the BF16/TF32 correlation.
#include "tc_internal.h"

namespace tc {

bool gram_tc_supported(int, int) { return false; }
void launch_gram_tc(tc_ctx*, const float*, const int32_t*, const int32_t*, int, int, int, float*, cudaStream_t) {
    throw TcError{TC_ERR_UNSUPPORTED, "tensor-core Gram not built"};
}
bool tc_assign_supported(int, int, int, int) { return false; }
void launch_assign_tc(tc_ctx*, const AssignArgs&, int, cudaStream_t) {
    throw TcError{TC_ERR_UNSUPPORTED, "tensor-core correlation not built"};
}

}  // namespace tc
