// Word-mask instances of the scan kernel, shared by es_scan_wm.cu (production launches) and
// es_scan_wmc.cu (counting launches): F in {0..6, 8}, inner rings of 1, 2, 3-4 or any words.
#pragma once
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
    if (words == 3 || words == 4) return pick_wm<COUNT, 4>(f);
    return pick_wm<COUNT, 0>(f);
}

}  // namespace
