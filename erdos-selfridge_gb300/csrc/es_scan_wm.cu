// Word-mask instances of the scan kernel for production launches (no stage counting).
#include "es_scan_wm.cuh"

ScanFn es_pick_wordmask_fast(uint32_t words, uint32_t f) { return pick_w<false>(words, f); }
