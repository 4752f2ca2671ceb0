// A host build of the segmented render's segment plan (seg_plan.h) for
// tests/test_seg_plan_cpu.py: the same function the device runs.
#include "seg_plan.h"

extern "C" int plan(const int *n, const int *end, const long long *px, long long budget, long long *out) {
    dmann::SegSpan sp[dmann::kSegSlots];
    const int ns = dmann::plan_segments(n, end, px, budget, sp);
    for (int i = 0; i < ns && i < dmann::kSegSlots; i++) {
        out[4 * i] = sp[i].lo;
        out[4 * i + 1] = sp[i].hi;
        out[4 * i + 2] = sp[i].stride;
        out[4 * i + 3] = sp[i].offset;
    }
    return ns;
}
