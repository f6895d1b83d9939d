// Scalar-layout instances of the scan kernel (runtime filter count up to 2, 4 or 8).
#include "es_scan_kernel.cuh"

ScanFn es_pick_scalar(int count, uint32_t f) {
    if (count) {
        if (f <= 2) return es_scan_kernel<2, ES_LAYOUT_SCALAR, true, 0>;
        if (f <= 4) return es_scan_kernel<4, ES_LAYOUT_SCALAR, true, 0>;
        return es_scan_kernel<8, ES_LAYOUT_SCALAR, true, 0>;
    }
    if (f <= 2) return es_scan_kernel<2, ES_LAYOUT_SCALAR, false, 0>;
    if (f <= 4) return es_scan_kernel<4, ES_LAYOUT_SCALAR, false, 0>;
    return es_scan_kernel<8, ES_LAYOUT_SCALAR, false, 0>;
}
