// buff_stream.cu -- host side of the register-streaming BUFF scan
// (buff_stream.cuh): the unit list of a column and the launch, which picks the
// kernel built for the column's most common chunk width (buff_stream_np0..4.cu;
// up to two byte planes: four CTAs per SM, else two).
#include "internal.h"

namespace ebi {

cudaError_t launch_buff_stream_np0(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);
cudaError_t launch_buff_stream_np1(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);
cudaError_t launch_buff_stream_np2(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);
cudaError_t launch_buff_stream_np3(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);
cudaError_t launch_buff_stream_np4(uint32_t tb, const QueryParams& q, const BuffChunkInfo* info, const uint2* units,
                                   uint32_t unit_base, uint32_t n_units, uint32_t upc, uint32_t grid, ScanTotals* T,
                                   QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s);

std::vector<uint2> buff_units(const std::vector<ChunkDesc>& chunks, std::vector<uint32_t>& first_unit) {
    std::vector<uint2> u;
    first_unit.assign(chunks.size() + 1, 0);
    for (uint32_t c = 0; c < chunks.size(); ++c) {
        first_unit[c] = static_cast<uint32_t>(u.size());
        for (uint32_t r = 0; r < chunks[c].n_rows; r += kBuffUnitRows) u.push_back(make_uint2(c, r));
    }
    first_unit[chunks.size()] = static_cast<uint32_t>(u.size());
    return u;
}

uint32_t buff_uniform_units(const std::vector<uint32_t>& first_unit) {
    const size_t n = first_unit.size() - 1;  // chunks
    if (n == 0) return 0;
    const uint32_t upc = first_unit[1] - first_unit[0];
    if (upc == 0) return 0;
    for (size_t c = 0; c + 1 < n; ++c)
        if (first_unit[c + 1] - first_unit[c] != upc) return 0;
    return first_unit[n] - first_unit[n - 1] <= upc ? upc : 0;
}

cudaError_t launch_buff_stream(const QueryParams& q, const BuffChunkInfo* info, const uint2* units, uint32_t unit_base,
                               uint32_t n_units, uint32_t upc, uint32_t bits, uint32_t sms, ScanTotals* T,
                               QueryResult* res, uint32_t frac, uint32_t fold, cudaStream_t s) {
    constexpr uint32_t kWarps = 8;  // per CTA
    const uint32_t np = bits / 8, tb = bits % 8;
    const uint32_t max_grid = (n_units + kWarps - 1) / kWarps;
    const uint32_t grid = sms * (np <= 2 ? 4 : 2);
    const uint32_t g = grid < max_grid ? grid : (max_grid ? max_grid : 1);
    if (g > kScanSlots) return cudaErrorInvalidConfiguration;
    switch (np) {
    case 0: return tb ? launch_buff_stream_np0(tb, q, info, units, unit_base, n_units, upc, g, T, res, frac, fold, s)
                      : cudaErrorInvalidValue;
    case 1: return launch_buff_stream_np1(tb, q, info, units, unit_base, n_units, upc, g, T, res, frac, fold, s);
    case 2: return launch_buff_stream_np2(tb, q, info, units, unit_base, n_units, upc, g, T, res, frac, fold, s);
    case 3: return launch_buff_stream_np3(tb, q, info, units, unit_base, n_units, upc, g, T, res, frac, fold, s);
    case 4: return launch_buff_stream_np4(tb, q, info, units, unit_base, n_units, upc, g, T, res, frac, fold, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace ebi
