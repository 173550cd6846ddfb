// graph_filter_tc.cu -- tcgen05 tensor-core distance filter (placeholder
// until the kernel lands).
#include "graph.cuh"

int filter_tc(mdet_ctx* ctx, const uint16_t*, const float*, uint32_t, const BlockMeta*, const uint16_t*, const float*,
              uint32_t, const BlockMeta*, bool, const DstarTable&, CandBuf) {
    return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "tensor-core filter not built");
}
