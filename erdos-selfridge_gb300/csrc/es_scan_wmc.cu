// Word-mask instances of the scan kernel for counting launches (per-stage pass counts).
#include "es_scan_wm.cuh"

ScanFn es_pick_wordmask_count(uint32_t words, uint32_t f) { return pick_w<true>(words, f); }
