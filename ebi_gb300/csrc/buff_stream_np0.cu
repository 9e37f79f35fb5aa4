// buff_stream_np0.cu -- the register-streaming BUFF scan kernels for columns whose
// most common chunk width is 1..7 bits: tail plane only (one kernel per tail width).
#include "buff_stream.cuh"

namespace ebi {

cudaError_t launch_buff_stream_np0(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s) {
    switch (tb) {
    case 1: return launch_stream_kernel<0, 1>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 2: return launch_stream_kernel<0, 2>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 3: return launch_stream_kernel<0, 3>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 4: return launch_stream_kernel<0, 4>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 5: return launch_stream_kernel<0, 5>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 6: return launch_stream_kernel<0, 6>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    case 7: return launch_stream_kernel<0, 7>(q, info, units, unit_base, n_units, upc, grid, T, res, frac, fold, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
