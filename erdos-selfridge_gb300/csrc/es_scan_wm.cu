// Word-mask instances of the scan kernel: F in {0..6, 8}, counting on/off, 1, 2 or any words.
#include "es_scan_kernel.cuh"

namespace {

template <bool COUNT, int WT>
ScanFn pick_wm(uint32_t f) {
    switch (f) {
        case 0: return es_scan_kernel<0, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 1: return es_scan_kernel<1, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 2: return es_scan_kernel<2, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 3: return es_scan_kernel<3, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 4: return es_scan_kernel<4, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 5: return es_scan_kernel<5, ES_LAYOUT_WORDMASK, COUNT, WT>;
        case 6: return es_scan_kernel<6, ES_LAYOUT_WORDMASK, COUNT, WT>;
        default: return es_scan_kernel<8, ES_LAYOUT_WORDMASK, COUNT, WT>;
    }
}

template <bool COUNT>
ScanFn pick_w(uint32_t words, uint32_t f) {
    if (words == 1) return pick_wm<COUNT, 1>(f);
    if (words == 2) return pick_wm<COUNT, 2>(f);
    return pick_wm<COUNT, 0>(f);
}

}  // namespace

ScanFn es_pick_wordmask(int count, uint32_t words, uint32_t f) {
    return count ? pick_w<true>(words, f) : pick_w<false>(words, f);
}
