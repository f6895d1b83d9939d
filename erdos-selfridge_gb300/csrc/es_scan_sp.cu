// Staged-pair-table instances of the scan kernel (the pair tables of the inner-stage filters
// staged in shared memory; inner rings of one or two words), production and counting launches.
#include "es_scan_kernel.cuh"

namespace {

template <bool COUNT, int WT>
ScanFn pick_sp(uint32_t f) {
    switch (f) {
        case 0: return es_scan_kernel<0, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 1: return es_scan_kernel<1, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 2: return es_scan_kernel<2, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 3: return es_scan_kernel<3, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 4: return es_scan_kernel<4, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 5: return es_scan_kernel<5, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        case 6: return es_scan_kernel<6, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
        default: return es_scan_kernel<8, ES_LAYOUT_SMEM_PAIR, COUNT, WT>;
    }
}

}  // namespace

// Only inner rings of exactly one or two words (every plan of the launch).
ScanFn es_pick_smem_pair(int count, uint32_t words, uint32_t f) {
    if (words == 1) return count ? pick_sp<true, 1>(f) : pick_sp<false, 1>(f);
    if (words == 2) return count ? pick_sp<true, 2>(f) : pick_sp<false, 2>(f);
    return nullptr;
}
