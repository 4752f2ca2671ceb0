// seg_plan.h -- the segmented render's segment plan (k_seg_plan in
// disc_seg.cu runs it on the device), in a header a host compiler also
// takes, so the plan is unit-tested on the CPU.
#pragma once

#ifdef __CUDACC__
#define DMANN_HD __host__ __device__
#else
#define DMANN_HD
#endif

namespace dmann {

// The items are sorted into kClasses octaves of their disc's deposit scale;
// a segment of deposits spans at most kClassSpan consecutive octaves and
// about kDepPerPix FP32 additions per pixel, with kSegSlots segments at most
// per chunk.
constexpr int kClasses = 256;
constexpr int kClassSpan = 2;
constexpr int kDepPerPix = 512;
constexpr int kSegSlots = 64;

// One segment of deposits: items lo + offset, lo + offset + stride, ... below
// hi of the sorted list.
struct SegSpan {
    long long lo, hi;
    int stride, offset;
};
static_assert(sizeof(SegSpan) == 24, "the segment buffer holds 24-byte spans");

// The segment plan from the per-octave histograms: n[c] items ending at slot
// end[c] of the sorted list (k_seg_sort leaves each octave's end slot), px[c]
// deposits.  Consecutive octaves are grouped while the group spans at most
// kClassSpan octaves and budget deposits; an octave with more than budget
// deposits is dealt round robin into ceil(px / budget) segments of its own.
// Class 0 (discs with no weighted deposits: single pixels, zero flux) is one
// segment.  At most kSegSlots segments: the budget doubles until the plan
// fits; should it reach 2^61 deposits (more than any chunk makes) with the
// plan still too long -- only a set whose deposit scales cover more than
// 2 kSegSlots octaves gets there -- the octave span doubles instead, so the
// loop ends.  Writes the spans and returns their count.
DMANN_HD inline int plan_segments(const int *n, const int *end, const long long *px, long long budget0,
                                  SegSpan *spans) {
    long long budget = budget0 < 1 ? 1 : budget0;
    int span = kClassSpan;
    for (;;) {
        int ns = 0;
        auto push = [&](long long lo, long long hi, int stride, int offset) {
            if (ns < kSegSlots) spans[ns] = SegSpan{lo, hi, stride, offset};
            ns++;
        };
        if (n[0] > 0) push((long long)end[0] - n[0], end[0], 1, 0);
        int c0 = -1;
        long long lo = 0, hi = 0, acc = 0;
        for (int c = 1; c < kClasses; ++c) {
            if (n[c] == 0) continue;
            const long long f = (long long)end[c] - n[c];
            if (px[c] > budget) {
                if (c0 >= 0) push(lo, hi, 1, 0);
                c0 = -1;
                acc = 0;
                long long m = (px[c] + budget - 1) / budget;
                if (m > n[c]) m = n[c];
                for (long long k = 0; k < m; ++k) push(f, end[c], (int)m, (int)k);
                continue;
            }
            if (c0 >= 0 && (c - c0 >= span || acc + px[c] > budget)) {
                push(lo, hi, 1, 0);
                c0 = -1;
                acc = 0;
            }
            if (c0 < 0) {
                c0 = c;
                lo = f;
            }
            hi = end[c];
            acc += px[c];
        }
        if (c0 >= 0) push(lo, hi, 1, 0);
        if (ns <= kSegSlots) return ns;
        if (budget < (1LL << 61)) budget *= 2;
        else span = span < kClasses ? 2 * span : kClasses;
    }
}

}  // namespace dmann
