// buff_stream_np3.cu -- the register-streaming BUFF scan kernels for columns whose
// most common chunk width has 3 byte planes (one kernel per tail width).
#include "buff_stream.cuh"

namespace ebi {

cudaError_t launch_buff_stream_np3(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s) {
    switch (tb) {
    case 0: return launch_stream_kernel<3, 0>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 1: return launch_stream_kernel<3, 1>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 2: return launch_stream_kernel<3, 2>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 3: return launch_stream_kernel<3, 3>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 4: return launch_stream_kernel<3, 4>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 5: return launch_stream_kernel<3, 5>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 6: return launch_stream_kernel<3, 6>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 7: return launch_stream_kernel<3, 7>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
