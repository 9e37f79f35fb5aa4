// buff_stream_np1.cu -- the register-streaming BUFF scan kernels for columns whose
// most common chunk width has 1 byte plane (one kernel per tail width).
#include "buff_stream.cuh"

namespace ebi {

cudaError_t launch_buff_stream_np1(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s) {
    switch (tb) {
    case 0: return launch_stream_kernel<1, 0>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 1: return launch_stream_kernel<1, 1>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 2: return launch_stream_kernel<1, 2>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 3: return launch_stream_kernel<1, 3>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 4: return launch_stream_kernel<1, 4>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 5: return launch_stream_kernel<1, 5>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 6: return launch_stream_kernel<1, 6>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 7: return launch_stream_kernel<1, 7>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
