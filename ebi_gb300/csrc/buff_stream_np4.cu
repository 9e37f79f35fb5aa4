// buff_stream_np4.cu -- the register-streaming BUFF scan kernels for columns whose
// most common chunk width has 4 byte planes (one kernel per tail width).
#include "buff_stream.cuh"

namespace ebi {

cudaError_t launch_buff_stream_np4(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s) {
    switch (tb) {
    case 0: return launch_stream_kernel<4, 0>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
