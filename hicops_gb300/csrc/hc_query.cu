// DSLIM query on the device (DSLIM_QuerySpectrum, source/core/dslim_query.cpp:515-842).
//
// Kernels, in launch order:
//   k_windows   one thread per (spectrum, length): the precursor window
//               [minlimit, maxlimit] of DSLIM_BinarySearch (dslim_query.cpp:854-994).
//   k_search    persistent CTAs, one spectrum at a time (work stealing):
//               for every length with a non-empty window, the candidate range
//               is cut into shared-memory scorecard tiles; the postings of every
//               (peak, bin) pair (dslim_query.cpp:617-676) are streamed with
//               coalesced loads from a per-pair cursor, and each posting adds
//               (count, intensity) to its candidate's packed 64-bit scorecard
//               word with one shared-memory atomic. A candidate enters the
//               qualifying list the moment its shared-peak count reaches
//               min_shp; listed candidates are scored (dslim_query.cpp:679-725)
//               into the 1002-bin histogram, cpsms and the top hit.
//   k_search<WIDE> the same for spectra whose packed words could overflow
//               (a count past 127): 2 x 64-bit words per candidate, exact FP64.
//   k_tailfit   one thread per spectrum: expeRT::ModelTailFit (expeRT.cpp:572-718)
//               and e(x) = 10^(mu*maxhyp + beta) * cpsms (dslim_query.cpp:773-799).
//
// Hyperscore. The reference evaluates h = lgfact[bc] + lgfact[yc] +
// log10(1+ibc) + log10(1+iyc) - 6 in double and stores it as float. Here it is
// first evaluated in float; the float value lies within 1.1e-4 of the
// reference's (table rounding 2 x 7.6e-6, three float additions 3 x 1.6e-5,
// log10f within 2 ulp, the final rounding 4e-6). Wherever that bound leaves a
// decision open (sign, histogram bin, or a candidate that can still be the
// top hit) the reference's double expression is evaluated, so cpsms, the
// histogram and the top hit equal the reference's double evaluation.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <cstdio>
#include <type_traits>

#include "hc_device.cuh"
#include "hc_internal.h"

namespace hc {
namespace {

constexpr int kDefer = HC_DEFER_MAX;  // undecided candidates per spectrum, resolved at its end
constexpr uint32_t kWQ = 128;        // per-warp ring of qualifying candidates (power of two, >= 32 + 64)
constexpr uint32_t kNoJob = 0xFFFFFFFFu;
constexpr float kApproxErr = 1.1e-4f;
constexpr float kBinMargin = 2.5e-3f;  // on the x10 scale: 10*(1.1e-4) + float product slack
constexpr float kNear = 3.5e-4f;       // > 2 * kApproxErr: candidates that may be the top
static_assert(HC_DEFER_MAX >= 128, "the scan's last step may read 127 packed words past the tile, into the queue");

// What the tile loop reads of a length's record: kept in the kernel's
// parameters (the constant cache; the length index is warp-uniform)
struct LenS
{
    const uint32_t *qp, *rows;  // search postings and their row table
    uint32_t stride, n;
    const uint8_t *cls;         // entry classes (4 bytes of padding past the last entry)
};

struct SearchArgs
{
    const LenDev *lens;
    uint32_t nlen;
    const QueryConst *qc;
    const uint32_t *idx, *moz, *inten;
    const float *prec;
    const int2 *win;
    uint32_t nspec;
    uint32_t dF, thr, min_shp, maxbin;  // maxbin = max_mass*scale
    hc_result *out;
    uint32_t *hist;
    uint32_t *wide_list, *nwide;
    uint32_t *work;
    uint32_t tile;
    uint32_t defer_cap;     // <= kDefer
    const uint32_t *only;   // optional list of spectra to process (wide pass)
    const uint32_t *nonly_dev;  // its length, in device memory
    const uint32_t *order;  // optional processing order (longest first)
    const uint32_t *obase;  // optional (device word): the first position of the order this launch takes
    const uint32_t *olim;   // optional (device word): the position it stops at (else nspec)
    uint32_t always_return; // the stream's atomics always return the old words (no all-pairs peak test)
    uint32_t persistent;    // 1: CTAs loop over a work counter; 0: one spectrum per CTA
    uint32_t maxz;
    const ClassKeys *classes;   // entry classes (null: none built)
    unsigned long long *phase;  // optional: SM cycles per phase, summed over CTAs (kPhases)
    LenS len[HC_MAX_LENGTHS];
};

// phases of k_search timed when SearchArgs::phase is set
constexpr int kPhases = 6;  // bucket setup | postings stream | score pass 1 | pass 2 | tile clear | rest

// The reference's double-precision hyperscore, rounded to float
// (dslim_query.cpp:695-698). Additions only: no contraction possible.
__device__ __forceinline__ float exact_h(const QueryConst *__restrict__ qc, uint32_t bc, uint32_t yc,
                                        uint64_t ib, uint64_t iy)
{
    const double h1 = __dadd_rn(qc->lgfact[bc < kLgTable ? bc : kLgTable - 1],
                                qc->lgfact[yc < kLgTable ? yc : kLgTable - 1]);
    // log10 of the intensity sums from the host-built table (the device's
    // double log10 is very slow on this part); beyond it, the device log10
    const double lb = (1 + ib < kLog10Tab) ? __ldg(qc->log10_tab + 1 + ib) : log10((double)(1 + ib));
    const double ly = (1 + iy < kLog10Tab) ? __ldg(qc->log10_tab + 1 + iy) : log10((double)(1 + iy));
    double h = __dadd_rn(h1, lb);
    h = __dadd_rn(h, ly);
    h = __dadd_rn(h, -6.0);
    return __double2float_rn(h);
}

template <bool WIDE>
struct Card;

template <>
struct Card<false>
{
    // b word [bc:8 | ibc:24] and y word [yc:8 | iyc:24]: a posting is a b or
    // a y ion, so it adds to one 32-bit word (native shared-memory atomic).
    // Every atomic returns the word before the add; a count that passes 128
    // shows as a returned top bit, and the spectrum is redone wide. Below
    // that, with intensities < 2^17, the sums stay below 2^24.
    using word = uint32_t;
    static constexpr int kWords = 2;
};

template <>
struct Card<true>
{
    // b word and y word: [count:24 | sum:40]
    using word = unsigned long long;
    static constexpr int kWords = 2;
};

// histogram bins kept in shared memory; candidates of the bins past them
// (hyperscores of 25.6 and more: a few per spectrum) add to the spectrum's
// output histogram directly
constexpr int kHistSm = 256;
// float log-factorials kept in shared memory: a packed count stays below 128
// (a spectrum whose count reaches 128 is redone with wide words)
constexpr int kLgSm = 128;

struct SmemTail
{
    union
    {
        // while the spectrum's candidates are scored; lgf first: an
        // overflowing packed count (up to 255, redone wide) reads histogram
        // words, inside the block's memory
        struct
        {
            float lgf[kLgSm];
            uint32_t hist[kHistSm];
        } run;
        // during the spectrum's set-up: per entry class, what its y1 keys
        // collect from the valid peaks as a wide word [count:24 | sum:40]
        // (kept apart for wide words, whose scorecard start reads it); the
        // valid peaks that can reach a class key
        struct
        {
            unsigned long long ucls[kMaxClasses + 1];
            uint32_t low[HC_QALEN];
        } setup;
    } u;
    unsigned long long best;   // (exact h bits << 32) | ~(ixx << 24 | psid)
    uint32_t best_shp;
    uint32_t maxbits;          // running max of the float estimate
    uint32_t cpsms;
    uint32_t qcount;
    uint32_t flags;
    uint32_t overflow;
    uint32_t spec;
    uint32_t nv;
    uint32_t noret;            // the stream's atomics need not return the old words (see k_search)
    uint32_t pnext;            // next 16-byte chunk (of the tile's lists laid end to end) to hand out
    uint32_t ndefer;           // undecided candidates queued for the exact evaluation
    uint32_t cchunks;          // 16-byte chunks (all lists) of the job
    uint32_t ncl;              // its non-empty lists
    unsigned long long bytes;
    unsigned long long ph[kPhases];
    unsigned long long ph_last;
    unsigned long long cnt[4];  // tiles | tiles scanned whole | listed candidates | exact evaluations
    int2 win[HC_MAX_LENGTHS];  // the spectrum's window per length
    uint32_t wtail[32];        // per warp: candidates appended to its ring so far (this job)
    // per entry class: what its y1 keys collect from the spectrum's valid
    // peaks, packed [count:8 | sum:24]; entry kClassNone stays zero
    uint32_t upk[kMaxClasses + 1];
    uint32_t nlow;
};

// adds the cycles since the last mark to phase k (thread 0 only, after a barrier)
#define HC_PHASE(k)                                               \
    do {                                                          \
        if (a.phase && tid == 0)                                  \
        {                                                         \
            const unsigned long long _t = clock64();              \
            T.ph[(k)] += _t - T.ph_last;                          \
            T.ph_last = _t;                                       \
        }                                                         \
    } while (0)

struct SmemLayout
{
    size_t qual, defer, lnext, lend, loff, coff, kinfo, pmoz, pint, wq, ucls, sink, tail, total;
    uint32_t maxpairs;  // lists: valid peaks x bins
};

__host__ __device__ inline SmemLayout smem_layout(uint32_t tile, uint32_t dF, bool wide, uint32_t nwarps)
{
    const size_t maxpairs = (size_t)HC_QALEN * (2 * dF + 1);
    SmemLayout o;
    // the scorecard, then the undecided queue: the scan reads whole
    // 128-candidate steps, and a window's last step may read up to 127 words
    // past the tile's end (masked), inside the queue
    o.qual = wide ? (size_t)tile * 16 : (size_t)tile * 8;
    o.defer = o.qual;
    o.maxpairs = (uint32_t)maxpairs;
    // per list (of the next job: written while the job streams): its first
    // posting, the end of its list, its chunk count; per non-empty list of
    // the job: its first chunk and {first posting, intensity} (the next
    // job's written after the job's stream)
    o.lnext = o.defer + 8ull * kDefer;
    o.lend = o.lnext + 4 * maxpairs;
    o.loff = o.lend + 4 * maxpairs;
    o.coff = o.loff + 4 * (maxpairs + 4);
    o.kinfo = (o.coff + 4 * (maxpairs + 4) + 7) & ~(size_t)7;
    o.pmoz = (o.kinfo + 8 * maxpairs + 15) & ~(size_t)15;
    o.pint = o.pmoz + 4ull * HC_QALEN;
    o.wq = (o.pint + 4ull * HC_QALEN + 15) & ~(size_t)15;
    size_t end = o.wq + 2ull * kWQ * nwarps;
    // wide words: the class adds, read by every job's scorecard start
    o.ucls = (end + 15) & ~(size_t)15;
    if (wide) end = o.ucls + 8ull * (kMaxClasses + 1);
    o.sink = (end + 15) & ~(size_t)15;
    o.tail = o.sink + 4 * 32;
    // right after the tail: per group of 32 lists of the next job, its chunks
    // and non-empty lists
    o.total = o.tail + sizeof(SmemTail) + 8 * ((maxpairs + 31) / 32);
    return o;
}

// float estimate of the hyperscore; the packed sums are < 2^24, so the
// integer-to-float conversions stay 32-bit (exact, full-rate). The two
// logarithms are one of the product (< 2^48, rounded by 2^-24 relative) with
// the fast hardware log2: together about 1e-6 off, well inside kApproxErr,
// which the callers' sign and bin margins are built on.
__device__ __forceinline__ float approx_h(const float *lgf, uint32_t bc, uint32_t yc, uint64_t ib, uint64_t iy)
{
    const float fb = __uint2float_rn((uint32_t)ib + 1u), fy = __uint2float_rn((uint32_t)iy + 1u);
    return (lgf[bc] + lgf[yc]) + __log2f(fb * fy) * 0.30102999566f - 6.0f;  // one log of the product
}

__device__ __forceinline__ void decode_packed(uint32_t wb, uint32_t wy, uint32_t &bc, uint32_t &yc, uint32_t &shp,
                                              uint64_t &ib, uint64_t &iy)
{
    bc = wb >> 24;
    yc = wy >> 24;
    ib = wb & 0xFFFFFFu;
    iy = wy & 0xFFFFFFu;
    shp = (uint32_t)(uint16_t)(bc + yc);
}

template <bool WIDE>
__device__ __forceinline__ void decode(const typename Card<WIDE>::word *card, uint32_t loc, uint32_t &bc,
                                       uint32_t &yc, uint32_t &shp, uint64_t &ib, uint64_t &iy)
{
    if constexpr (!WIDE)
    {
        const uint2 w = *reinterpret_cast<const uint2 *>(card + 2 * loc);
        decode_packed(w.x, w.y, bc, yc, shp, ib, iy);
        return;
    }
    else
    {
        const unsigned long long wb = card[2 * loc], wy = card[2 * loc + 1];
        bc = (uint32_t)(wb >> 40);
        yc = (uint32_t)(wy >> 40);
        ib = wb & 0xFFFFFFFFFFull;
        iy = wy & 0xFFFFFFFFFFull;
    }
    // the reference reads bc/yc through short/ushort (dslim_query.cpp:684-686)
    shp = (uint32_t)(uint16_t)(bc + yc);
}

// Hyperscore of one candidate: returns false unless h > 0; h is the float
// estimate (or the reference's value where the estimate's bound leaves the
// sign or the histogram bin undecided), bin its histogram bin.
template <bool WIDE>
__device__ __forceinline__ bool score(const QueryConst *__restrict__ qc, const float *lgf, uint32_t bc, uint32_t yc,
                                      uint64_t ib, uint64_t iy, float &h, int &bin, uint32_t &nexact)
{
    if (!WIDE)
    {
        const float ha = approx_h(lgf, bc, yc, ib, iy);
        const float t = ha * 10.0f + 0.5f;
        const float fr = t - floorf(t);
        if (!(fabsf(ha) <= kApproxErr * 4.0f || fr < kBinMargin || fr > 1.0f - kBinMargin))
        {
            h = ha;
            bin = (int)floorf(t);
            return ha > 0.0f;
        }
    }
    nexact++;
    const float hf = exact_h(qc, bc, yc, ib, iy);
    h = hf;
    bin = hist_bin(hf);
    return hf > 0.0f;
}

// 32-bit adds to a shared-memory word given by its shared-window address.
// No memory clobber: the scorecard is read only after a block barrier.
__device__ __forceinline__ void red_shared_add(uint32_t addr, uint32_t v)
{
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(v));
}

__device__ __forceinline__ uint32_t atom_shared_add(uint32_t addr, uint32_t v)
{
    uint32_t old;
    asm volatile("atom.shared.add.u32 %0, [%1], %2;" : "=r"(old) : "r"(addr), "r"(v));
    return old;
}

// Bounds of a bucket's postings for candidates [c0, c1), widened to row-table
// boundaries (multiples of kRowG entries): the postings of entries outside
// the range are read but fail the scorecard's index test, so no search is
// needed. Tile boundaries inside a window are multiples of kRowG already.
__device__ __forceinline__ uint32_t row_lo(const uint32_t *__restrict__ col, uint32_t c0)
{
    return __ldg(col + c0 / kRowG);
}

__device__ __forceinline__ uint32_t row_hi(const uint32_t *__restrict__ col, uint32_t c1)
{
    return __ldg(col + (c1 + kRowG - 1) / kRowG);
}

// Chunk offsets of a job's lists, in two steps around a block barrier, with
// the lists in groups of 32 (group g = lists 32g .. 32g + 31).
// Step 1, by the warp that computed the group's chunk counts (cnt = this
// lane's list, 0 past the last list): the group's totals of chunks and of
// non-empty lists.
__device__ __forceinline__ void group_totals(uint32_t cnt, uint32_t g, int lane, uint2 *gt)
{
    const uint32_t c = __reduce_add_sync(0xFFFFFFFFu, cnt);
    const uint32_t z = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, cnt != 0u));
    if (lane == 0) gt[g] = make_uint2(c, z);
}

// Step 2, one warp per group, any warp: from the chunk counts lo[0, np) and
// the group totals, the job's non-empty lists in order: coff[k] = its first
// chunk (of all lists laid end to end), kinfo[k] = {its first posting, its
// peak's intensity} (list pr = peak pr / nbin, bin pr % nbin); the warp of
// the last group (of ng) writes coff[ncl] = *total and the counts.
__device__ __forceinline__ void group_offsets(uint32_t g, uint32_t ng, const uint32_t *lo, uint32_t np, int lane,
                                              const uint2 *gt, const uint32_t *first, const uint32_t *pint,
                                              uint32_t nbin, uint32_t *coff, uint2 *kinfo, uint32_t *total,
                                              uint32_t *ncl)
{
    uint32_t pc = 0, pz = 0;
    for (uint32_t i = (uint32_t)lane; i < g; i += 32)
    {
        const uint2 t = gt[i];
        pc += t.x;
        pz += t.y;
    }
    pc = __reduce_add_sync(0xFFFFFFFFu, pc);
    pz = __reduce_add_sync(0xFFFFFFFFu, pz);
    const uint32_t pr = 32 * g + (uint32_t)lane;
    const uint32_t cnt = pr < np ? lo[pr] : 0u;
    uint32_t c = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, c, o);
        if (lane >= o) c += y;
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, cnt != 0u);
    if (cnt)
    {
        const uint32_t k = pz + (uint32_t)__popc(bal & ((1u << lane) - 1u));
        coff[k] = pc + c - cnt;
        kinfo[k] = make_uint2(first[pr], pint[pr / nbin]);
    }
    if (g + 1 == ng && lane == 31)
    {
        const uint32_t nz = pz + (uint32_t)__popc(bal);
        coff[nz] = pc + c;
        *total = pc + c;
        *ncl = nz;
    }
}

// One unit of a spectrum's work: the candidates [c0, c1) of length l, at
// most one scorecard tile. A window's first tile ends one tile past the
// window start rounded down to a row-table boundary (kRowG); every later
// boundary is a multiple of kRowG, so only a window's two ends widen the
// postings bounds.
struct Job
{
    uint32_t l, c0, c1;
};

__device__ __forceinline__ Job job_from(const int2 *win, uint32_t nlen, uint32_t tile, uint32_t l)
{
    for (; l < nlen; l++)
    {
        const int2 w = win[l];
        if (w.x <= w.y)
        {
            const uint32_t c0 = (uint32_t)w.x;
            return Job{l, c0, min((uint32_t)w.y + 1, (c0 / kRowG) * kRowG + tile)};
        }
    }
    return Job{kNoJob, 0u, 0u};
}

__device__ __forceinline__ Job first_job(const int2 *win, uint32_t nlen, uint32_t tile)
{
    return job_from(win, nlen, tile, 0);
}

__device__ __forceinline__ Job next_job(const Job &j, const int2 *win, uint32_t nlen, uint32_t tile)
{
    const uint32_t end = (uint32_t)win[j.l].y + 1;
    if (j.c1 < end) return Job{j.l, j.c1, min(end, j.c1 + tile)};
    return job_from(win, nlen, tile, j.l + 1);
}

// A job whose bounds are both row-table boundaries inside the length's
// entries: its lists hold the postings of the job's entries and nothing else
// (no padding, no neighbours), so their lengths are its visited postings.
__device__ __forceinline__ bool job_interior(const Job &j, uint32_t n)
{
    return (j.c0 % kRowG) == 0 && (j.c1 % kRowG) == 0 && j.c1 < n;
}

// The last list i in [0, n) with off[i] <= q (off ascending, off[0] = 0):
// a 32-way search, one shared-memory read per lane per round.
__device__ __forceinline__ uint32_t find_list(const uint32_t *off, uint32_t n, uint32_t q, int lane)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1)
    {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t i = lo + (uint32_t)lane * step;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, i < hi && off[i] <= q);
        lo += (uint32_t)(31 - __clz(m)) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}

template <bool WIDE, int G>
__global__ void __launch_bounds__(G >= 4 ? 512 : 1024, G == 4 ? 2 : 1) k_search(SearchArgs a)
{
    using W = typename Card<WIDE>::word;
    constexpr int NW = Card<WIDE>::kWords;
    // lists per thread whose bucket is kept and whose next-job row-table
    // words are loaded early (two for blocks of up to 512 threads, one for
    // 1024: 300 lists at dF = 1 either way; the rest are computed directly)
    constexpr int kPf = G >= 4 ? 2 : 1;
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t tile = a.tile;
    const uint32_t nbin = 2 * a.dF + 1;
    const SmemLayout L = smem_layout(tile, a.dF, WIDE, blockDim.x >> 5);
    W *card = reinterpret_cast<W *>(smem);
    uint32_t *coff = reinterpret_cast<uint32_t *>(smem + L.coff);    // first chunk of each non-empty list
    uint2 *kinfo = reinterpret_cast<uint2 *>(smem + L.kinfo);         // {first posting, intensity} of each
    uint2 *defer = reinterpret_cast<uint2 *>(smem + L.defer);  // undecided candidates: {b word, y word}
    uint32_t *lnext = reinterpret_cast<uint32_t *>(smem + L.lnext);  // per list: first posting (next job)
    uint32_t *lend = reinterpret_cast<uint32_t *>(smem + L.lend);  // per list: end of the current job's list
    uint32_t *loff = reinterpret_cast<uint32_t *>(smem + L.loff);
    uint32_t *pmoz = reinterpret_cast<uint32_t *>(smem + L.pmoz);
    uint32_t *pint = reinterpret_cast<uint32_t *>(smem + L.pint);
    SmemTail &T = *reinterpret_cast<SmemTail *>(smem + L.tail);
    uint2 *gt = reinterpret_cast<uint2 *>(&T + 1);
    unsigned long long *ucls = WIDE ? reinterpret_cast<unsigned long long *>(smem + L.ucls) : T.u.setup.ucls;
    uint32_t *low = T.u.setup.low;

    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5;
    // one word per lane that postings outside the tile add to (never read);
    // the stream addresses the scorecard and the sinks as shared-window offsets
    const uint32_t card_s = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t sink_s = (uint32_t)__cvta_generic_to_shared(smem + L.sink) + 4u * (uint32_t)lane;
    uint16_t *wq = reinterpret_cast<uint16_t *>(smem + L.wq) + wid * kWQ;  // this warp's candidate ring (tile < 2^16)

    for (uint32_t i = tid; i < tile * NW; i += nthr) card[i] = 0;
    if (tid == 0)
    {
        for (int k = 0; k < kPhases; k++) T.ph[k] = 0;
        for (int k = 0; k < 4; k++) T.cnt[k] = 0;
        T.ph_last = clock64();
        T.pnext = 0;   // reset again after every tile
        T.qcount = 0;
    }

    // Scores one candidate (the float estimate; undecided ones are queued):
    // cpsms, histogram, flags. A candidate whose estimate comes within kNear
    // of the running maximum (all candidates of the spectrum so far) gets the
    // reference's double hyperscore and competes for the top hit. The true top
    // hit's estimate is within 2*kApproxErr < kNear of the final maximum, so it
    // is always among them, whatever the order candidates are scored in.
    uint32_t my_cps = 0, my_fl = 0, my_exact = 0;
    auto hist_add = [&](int bin) {
        if (bin < kHistSm) atomicAdd(&T.u.run.hist[bin], 1u);
        else atomicAdd(&a.hist[(size_t)T.spec * HC_HIST_BINS + (uint32_t)bin], 1u);
    };
    unsigned long long my_best = 0;
    uint32_t my_shp = 0;
    auto score_one = [&](uint32_t bc, uint32_t yc, uint64_t ib, uint64_t iy, uint32_t shp, uint32_t key_lo) {
        float ha;
        if constexpr (!WIDE) ha = approx_h(T.u.run.lgf, bc, yc, ib, iy);
        else ha = exact_h(a.qc, bc, yc, ib, iy);
        const float runmax = __uint_as_float(*(volatile uint32_t *)&T.maxbits);
        if (ha >= runmax - kNear)
        {
            if (ha > runmax) atomicMax(&T.maxbits, __float_as_uint(ha));
            const float he = WIDE ? ha : exact_h(a.qc, bc, yc, ib, iy);
            if (he > 0.0f)
            {
                const unsigned long long key = ((unsigned long long)__float_as_uint(he) << 32) | key_lo;
                if (key > my_best)
                {
                    my_best = key;
                    my_shp = shp;
                }
                atomicMax(&T.best, key);
            }
        }
        float h;
        int bin;
        if constexpr (!WIDE)
        {
            const float tt = ha * 10.0f + 0.5f;
            const float fr = tt - floorf(tt);
            if (fabsf(ha) <= kApproxErr * 4.0f || fr < kBinMargin || fr > 1.0f - kBinMargin)
            {
                const uint32_t di = atomicAdd(&T.ndefer, 1u);
                if (di < a.defer_cap)
                {
                    defer[di] = make_uint2((uint32_t)ib | (bc << 24), (uint32_t)iy | (yc << 24));
                    return;
                }
                my_exact++;  // queue full: exact now
                h = exact_h(a.qc, bc, yc, ib, iy);
                bin = hist_bin(h);
                if (!(h > 0.0f)) return;
            }
            else
            {
                if (!(ha > 0.0f)) return;
                h = ha;
                bin = (int)floorf(tt);
            }
        }
        else
        {
            my_exact++;
            h = ha;
            bin = hist_bin(h);
            if (!(h > 0.0f)) return;
        }
        my_cps++;
        if (bc >= (uint32_t)kRefMaxShp || yc >= (uint32_t)kRefMaxShp) my_fl |= HC_FLAG_LGFACT_OOB;
        if (bin >= HC_HIST_BINS || bin < 0) { my_fl |= HC_FLAG_HIST_OOB; bin = bin < 0 ? 0 : HC_HIST_BINS - 1; }
        hist_add(bin);
    };

    for (uint32_t iter = 0;; iter++)
    {
        __syncthreads();
        if (tid == 0)
        {
            const uint32_t w = a.persistent ? atomicAdd(a.work, 1u) : (iter == 0 ? blockIdx.x : 0xFFFFFFFFu);
            uint32_t sp = 0xFFFFFFFFu;
            if (a.only) sp = w < *a.nonly_dev ? a.only[w] : 0xFFFFFFFFu;
            else
            {
                const uint32_t o = (a.obase ? *a.obase : 0u) + w;
                if (w < a.nspec && o < (a.olim ? *a.olim : a.nspec)) sp = a.order ? a.order[o] : o;
            }
            T.spec = sp;
        }
        __syncthreads();
        const uint32_t s = T.spec;
        if (s == 0xFFFFFFFFu) break;
        for (int i = kHistSm + tid; i < HC_HIST_BINS; i += nthr) a.hist[(size_t)s * HC_HIST_BINS + i] = 0;
        if (tid == 0)
        {
            T.best = 0;
            T.best_shp = 0;
            T.maxbits = 0;
            T.cpsms = 0;
            T.qcount = 0;
            T.ndefer = 0;
            T.flags = WIDE ? HC_FLAG_WIDE : 0u;
            T.overflow = 0;
            T.bytes = 0;
            T.nv = 0;
            T.nlow = 0;
        }
        for (uint32_t l = tid; l < a.nlen; l += nthr) T.win[l] = a.win[(size_t)s * a.nlen + l];
        for (uint32_t i = tid; i < kMaxClasses + 1; i += nthr) ucls[i] = 0ull;
        __syncthreads();
        // valid peaks (dslim_query.cpp:625): dF < qion < max*scale - 1 - dF
        {
            const uint32_t lowlim = a.classes ? __ldg(&a.classes->maxkey) + a.dF : 0u;
            const uint32_t p0 = a.idx[s], p1 = a.idx[s + 1];
            for (uint32_t k = p0 + tid; k < p1; k += nthr)
            {
                const uint32_t q = a.moz[k];
                if (q > a.dF && (uint64_t)q + 1 + a.dF < a.maxbin)
                {
                    // packed sums stay exact only for intensities below 2^17
                    if (!WIDE && a.inten[k] >= (1u << 17)) T.overflow = 1;
                    const uint32_t slot = atomicAdd(&T.nv, 1u);
                    if (slot < HC_QALEN)
                    {
                        pmoz[slot] = q;
                        pint[slot] = a.inten[k];
                        if (q <= lowlim) low[atomicAdd(&T.nlow, 1u)] = slot;
                    }
                }
            }
        }
        __syncthreads();
        const uint32_t nv = T.nv < HC_QALEN ? T.nv : HC_QALEN;
        // The stream's atomics need not return the old words when no word can
        // reach a count of 128: if every list of the spectrum has a bucket of
        // its own (valid peaks more than 2*dF bins apart), a candidate's b (y)
        // count is at most its number of b (y) ions, (L-1)*maxz, below 128 for
        // every length; with intensities below 2^17 the sums stay below 2^24.
        // (The small-window launch skips the all-pairs test: its spectra visit
        // few postings, so returning atomics cost less than the test.)
        if (!WIDE && a.always_return)
        {
            if (tid == 0) T.noret = 0u;
        }
        else if constexpr (!WIDE)
        {
            // warp w takes peaks i = w, w + nw, ...; its lanes the peaks j > i
            bool close = false;
            for (uint32_t i = (uint32_t)wid; i < nv; i += (uint32_t)(nthr >> 5))
            {
                const uint32_t x = pmoz[i];
                for (uint32_t j = i + 1 + (uint32_t)lane; j < nv; j += 32)
                {
                    const uint32_t y = pmoz[j];
                    close |= (x > y ? x - y : y - x) <= 2 * a.dF;
                }
            }
            close = __syncthreads_or(close);
            if (tid == 0) T.noret = (!close && a.lens[a.nlen - 1].half < 128u) ? 1u : 0u;
        }
        // the class adds: for each class, charge and valid peak whose bins
        // (q - dF .. q + dF) hold the class's y1 key, what the left-out
        // posting of every entry of the class would add there
        if (a.classes)
        {
            const uint32_t nz = a.maxz, tot = a.classes->n * nz, nlow = T.nlow;
            for (uint32_t i = tid; i < tot; i += nthr)
            {
                const uint32_t c = i / nz, z = i - c * nz;
                const uint32_t key = a.classes->key[c][z];
                unsigned long long acc = 0;
                for (uint32_t t = 0; t < nlow; t++)
                {
                    const uint32_t sl = low[t], q = pmoz[sl];
                    if (q <= key + a.dF && q + a.dF >= key) acc += (1ull << 40) | pint[sl];
                }
                if (acc) atomicAdd(&ucls[c], acc);
            }
        }
        __syncthreads();
        for (uint32_t i = tid; i < kMaxClasses + 1; i += nthr)
        {
            // packed: a count of 64 or more from a class alone is redone wide
            const unsigned long long u = ucls[i];
            if (!WIDE && (u >> 40) >= 64u) T.overflow = 1;
            T.upk[i] = ((uint32_t)(u >> 40) << 24) | (uint32_t)(u & 0xFFFFFFull);
        }
        __syncthreads();
        // the set-up's tables are read: their space takes the scoring's (seen
        // by the scan after the first job's barriers)
        for (int i = tid; i < kLgSm; i += nthr) T.u.run.lgf[i] = a.qc->lgfact_f[i];
        for (int i = tid; i < kHistSm; i += nthr) T.u.run.hist[i] = 0;
        const uint32_t np = nv * nbin;
        my_best = 0;
        my_shp = 0;
        if (tid == 0)
            for (uint32_t l = 0; l < a.nlen; l++)
                if (T.win[l].x <= T.win[l].y) atomicAdd(&T.bytes, 4ull * (2 * a.dF + 2) * nv);  // the reference's bA reads

        // The spectrum's work is a sequence of jobs (length l, scorecard tile
        // t). Interior tile boundaries are row-table entries; a window's own
        // ends are widened to the nearest ones (see row_lo / row_hi). The
        // per-list bounds are pipelined: while job j streams, the row-table
        // words of job j+1's boundaries are in flight; right after its own
        // stream each thread turns them into job j+1's bounds (lnext, lend,
        // loff), and after the barrier that ends the stream the warps turn
        // those into job j+1's chunk offsets and {first posting, intensity}
        // per non-empty list, which only job j+1's stream reads. (Asking L2
        // for job j+1's postings at that point was measured: it cost more
        // issue slots than the latency it hid.)
        Job jb = first_job(T.win, a.nlen, tile);
        uint32_t pf_hi[kPf], ps_lo[kPf];
        // the bucket and the intensity of this thread's lists tid + m * nthr
        // (list = (valid peak, bin)): the same for every job of the spectrum
        uint32_t my_bkt[kPf];
#pragma unroll
        for (int m = 0; m < kPf; m++)
        {
            const uint32_t pr = tid + m * nthr;
            my_bkt[m] = 0u;
            if (pr < np)
            {
                const uint32_t k = pr / nbin, j = pr - k * nbin;
                my_bkt[m] = pmoz[k] - a.dF + j;
            }
        }
        uint32_t npass = 0;  // postings of entries inside the window (the reference visits exactly these)
        const uint32_t nw = (uint32_t)nthr >> 5, ng = (np + 31) >> 5;
        if (jb.l != kNoJob)
        {
            // the first job's boundaries, directly
            const LenS d = a.len[jb.l];
            const bool inter = !WIDE && job_interior(jb, d.n);
            for (uint32_t base = 0; base < np; base += (uint32_t)nthr)
            {
                const uint32_t pr = base + (uint32_t)tid;
                uint32_t cnt = 0;
                if (pr < np)
                {
                    const uint32_t k = pr / nbin, j = pr - k * nbin;
                    const uint32_t *col = d.rows + (size_t)(pmoz[k] - a.dF + j) * d.stride;
                    const uint32_t st = row_lo(col, jb.c0), en = row_hi(col, jb.c1);
                    if (inter && st < en) npass += en - st;
                    lnext[pr] = st;
                    lend[pr] = en;
                    cnt = st < en ? ((en + 3) >> 2) - (st >> 2) : 0u;
                    loff[pr] = cnt;
                }
                if (base + 32 * (uint32_t)wid < np) group_totals(cnt, (pr >> 5), lane, gt);
            }
            // the first job's scorecard: each candidate's y word starts with its class's adds
            {
                const uint32_t nt0 = jb.c1 - jb.c0;
                const uint8_t *cl0 = d.cls + jb.c0;
                for (uint32_t c = tid; c < nt0; c += nthr)
                {
                    const uint32_t k = __ldg(cl0 + c);
                    if constexpr (!WIDE)
                    {
                        const uint32_t wy = T.upk[k];
                        card[2 * c + 1] = wy;
                        npass += wy >> 24;
                    }
                    else
                    {
                        const W wy = ucls[k];
                        card[2 * c + 1] = wy;
                        npass += (uint32_t)(wy >> 40);
                    }
                }
            }
            __syncthreads();
            for (uint32_t g = nw - 1 - (uint32_t)wid; g < ng; g += nw)
                group_offsets(g, ng, loff, np, lane, gt, lnext, pint, nbin, coff, kinfo, &T.cchunks, &T.ncl);
            if (ng == 0 && tid == 0) T.cchunks = T.ncl = coff[0] = 0;
        }
        __syncthreads();
        while (jb.l != kNoJob)
        {
            const LenS d = a.len[jb.l];
            const uint32_t c0 = jb.c0, ntile = jb.c1 - jb.c0;
            const uint32_t C = T.cchunks;
            const uint32_t ncl = T.ncl;
            const uint32_t *co = coff;
            HC_PHASE(0);
            // ---- row-table words of the next job's boundaries, in flight ----
            const Job nj = next_job(jb, T.win, a.nlen, tile);
            const bool same = nj.l == jb.l;
            LenS dn;
            if (nj.l != kNoJob)
            {
                dn = same ? d : a.len[nj.l];
#pragma unroll
                for (int m = 0; m < kPf; m++)
                {
                    const uint32_t pr = tid + m * nthr;
                    if (pr < np)
                    {
                        const uint32_t *col = dn.rows + (size_t)my_bkt[m] * dn.stride;
                        pf_hi[m] = row_hi(col, nj.c1);
                        if (!same) ps_lo[m] = row_lo(col, nj.c0);
                    }
                }
            }
            // ---- stream the job's postings into the scorecard ----
            // A warp takes 32*G consecutive chunks; lane j handles chunks
            // q0 + j + 32g. All G loads are issued before any is used. A
            // posting is the byte offset of its scorecard word counted from
            // entry 0, so one subtraction gives its place in the tile and one
            // unsigned compare rejects entries outside the tile and padding.
            // Visited postings are counted per posting only in a window's end
            // tiles; an interior tile's lists hold exactly the tile's entries,
            // and their lengths were added when its bounds were set.
            uint32_t ovf = 0;  // OR of the words the atomics returned
            auto stream = [&](auto no_return, auto count) {
            constexpr bool NR = decltype(no_return)::value;
            constexpr bool CNT = decltype(count)::value;
            (void)NR;
            (void)CNT;
            // packed: byte offsets of the tile's words; wide: word indexes
            [[maybe_unused]] const uint32_t base8 = c0 << kQpEntryShift, lim8 = ntile << kQpEntryShift;
            [[maybe_unused]] const uint32_t base2 = 2 * c0, lim2 = 2 * ntile;
            for (;;)
            {
                uint32_t q0 = 0;
                if (lane == 0) q0 = atomicAdd(&T.pnext, 32u * G);
                q0 = __shfl_sync(0xFFFFFFFFu, q0, 0);
                if (q0 >= C) break;
                uint4 v[G];
                uint32_t inte[G];
                // the list holding chunk q0, then for each group of 32 chunks the
                // list of every lane's chunk: lists that start inside the group
                // set one bit each at their first lane, and a lane's list is the
                // one before plus the bits at or below it
                uint32_t k0 = find_list(co, ncl, q0, lane);
                if (co[k0 + 1u] >= q0 + 32u * G)  // warp-uniform: the whole grab lies in list k0
                {
                    const uint2 ki = kinfo[k0];
                    const uint32_t p0 = (ki.x & ~3u) + 4u * (q0 + (uint32_t)lane - co[k0]);
                    const uint32_t li = ki.y;
#pragma unroll
                    for (int g = 0; g < G; g++)
                    {
                        inte[g] = li;
                        v[g] = __ldg(reinterpret_cast<const uint4 *>(d.qp + p0 + 128u * g));
                    }
                }
                else
#pragma unroll
                for (int g = 0; g < G; g++)
                {
                    const uint32_t kb = q0 + 32u * g;
                    const uint32_t kc = kb + (uint32_t)lane;
                    inte[g] = 0u;
                    v[g] = make_uint4(kQpostPad, kQpostPad, kQpostPad, kQpostPad);
                    if (kb < C && co[k0 + 1u] >= kb + 32u)  // warp-uniform
                    {
                        // the group's 32 chunks all lie in list k0 (most
                        // postings sit in long lists): one lookup for the warp
                        const uint2 ki = kinfo[k0];
                        const uint32_t pos = (ki.x & ~3u) + 4u * (kc - co[k0]);
                        inte[g] = ki.y;
                        v[g] = __ldg(reinterpret_cast<const uint4 *>(d.qp + pos));
                    }
                    else if (kb < C)  // warp-uniform
                    {
                        const uint32_t j1 = k0 + 1u + (uint32_t)lane;
                        const uint32_t u = (j1 <= ncl ? co[j1] : 0xFFFFFFFFu) - kb;  // >= 1
                        const uint32_t msk = __reduce_or_sync(0xFFFFFFFFu, u < 32u ? (1u << u) : 0u);
                        const uint32_t k = k0 + (uint32_t)__popc(msk & ((2u << lane) - 1u));
                        if (kc < C)
                        {
                            const uint2 ki = kinfo[k];
                            // a chunk never leaves its bucket (buckets start at
                            // multiples of 4, padded to them); its postings
                            // outside [first, end) belong to entries outside
                            // the tile and fail the index test below
                            const uint32_t pos = (ki.x & ~3u) + 4u * (kc - co[k]);
                            inte[g] = ki.y;
                            v[g] = __ldg(reinterpret_cast<const uint4 *>(d.qp + pos));
                        }
                        k0 = __shfl_sync(0xFFFFFFFFu, k, 31);  // the list holding chunk kb + 31
                    }
                }
#pragma unroll
                for (int g = 0; g < G; g++)
                {
                    const uint32_t xs[4] = {v[g].x, v[g].y, v[g].z, v[g].w};
                    if constexpr (!WIDE)
                    {
                        const uint32_t add = (1u << 24) | inte[g];
#pragma unroll
                        for (int e = 0; e < 4; e++)
                        {
                            // byte offset of the word in the tile; a posting
                            // outside the tile (or padding) adds to the lane's
                            // own sink word instead, so the atomic is not
                            // behind a branch
                            const uint32_t o = xs[e] - base8;
                            const bool in = o < lim8;
                            const uint32_t wa = in ? card_s + o : sink_s;
                            if constexpr (NR) red_shared_add(wa, add);
                            else
                            {
                                const uint32_t old = atom_shared_add(wa, add);
                                ovf |= in ? old : 0u;
                            }
                            if constexpr (CNT) npass += in ? 1u : 0u;
                        }
                    }
                    else
                    {
                        const W add = (1ull << 40) | (W)inte[g];
#pragma unroll
                        for (int e = 0; e < 4; e++)
                        {
                            const uint32_t w = (xs[e] >> 2) - base2;  // 2*(entry - c0) + isY
                            if (w < lim2)
                            {
                                atomicAdd(&card[w], add);
                                npass++;
                            }
                        }
                    }
                }
            }
            };
            if constexpr (WIDE) stream(std::false_type{}, std::true_type{});
            else
            {
                const bool cnt = !job_interior(jb, d.n);
                if (T.noret)
                {
                    if (cnt) stream(std::true_type{}, std::true_type{});
                    else stream(std::true_type{}, std::false_type{});
                }
                else
                {
                    if (cnt) stream(std::false_type{}, std::true_type{});
                    else stream(std::false_type{}, std::false_type{});
                }
            }
            if (!WIDE && (__reduce_or_sync(0xFFFFFFFFu, ovf) & 0x80000000u) && lane == 0) T.overflow = 1;
            // ---- the next job's list bounds ----
            if (nj.l != kNoJob)
            {
                const bool inter = !WIDE && job_interior(nj, dn.n);
#pragma unroll
                for (int m = 0; m < kPf; m++)
                {
                    const uint32_t pr = tid + m * nthr;
                    uint32_t cnt = 0, st = 0, en = 0;
                    if (pr < np)
                    {
                        st = same ? lend[pr] : ps_lo[m];
                        en = pf_hi[m];
                        if (inter && st < en) npass += en - st;
                        lnext[pr] = st;
                        lend[pr] = en;
                        cnt = st < en ? ((en + 3) >> 2) - (st >> 2) : 0u;
                        loff[pr] = cnt;
                    }
                    if (m * nthr + 32 * wid < np) group_totals(cnt, pr >> 5, lane, gt);
                }
                // lists past kPf * nthr (small blocks, wide bin windows): directly
                for (uint32_t base = kPf * nthr; base < np; base += (uint32_t)nthr)
                {
                    const uint32_t pr = base + (uint32_t)tid;
                    uint32_t cnt = 0, st = 0, en = 0;
                    if (pr < np)
                    {
                        const uint32_t k = pr / nbin, j = pr - k * nbin;
                        const uint32_t *col = dn.rows + (size_t)(pmoz[k] - a.dF + j) * dn.stride;
                        st = same ? lend[pr] : row_lo(col, nj.c0);
                        en = row_hi(col, nj.c1);
                        if (inter && st < en) npass += en - st;
                        lnext[pr] = st;
                        lend[pr] = en;
                        cnt = st < en ? ((en + 3) >> 2) - (st >> 2) : 0u;
                        loff[pr] = cnt;
                    }
                    if (base + 32 * (uint32_t)wid < np) group_totals(cnt, pr >> 5, lane, gt);
                }
            }
            __syncthreads();
            HC_PHASE(1);
            // ---- the next job's chunk offsets (one group of 32 lists per warp,
            // the last warps first: the first warps computed the bounds) ----
            if (nj.l != kNoJob)
            {
                for (uint32_t g = nw - 1 - (uint32_t)wid; g < ng; g += nw)
                    group_offsets(g, ng, loff, np, lane, gt, lnext, pint, nbin, coff, kinfo, &T.cchunks, &T.ncl);
                if (ng == 0 && tid == 0) T.cchunks = T.ncl = coff[0] = 0;
            }
            // ---- every candidate that reached min_shp ----
            // cpsms, histogram and the top hit (see score_one). The packed tile
            // is scanned two candidates per lane and step; a warp collects its
            // qualifying candidates in its own ring and scores them 32 at a
            // time (all lanes busy), then clears the words it scanned.
            my_cps = my_fl = my_exact = 0;
            const uint32_t key_l = jb.l << 24;
            if constexpr (!WIDE)
            {
                const uint4 *c4 = reinterpret_cast<const uint4 *>(card);
                uint32_t qh = 0, qhead = 0;  // ring fill and head (warp-uniform)
                if (lane == 0) T.wtail[wid] = 0;
                __syncwarp();
                auto pop_score = [&](uint32_t cnt) {
                    __syncwarp();
                    if ((uint32_t)lane < cnt)
                    {
                        const uint32_t loc = wq[(qhead + lane) & (kWQ - 1)];
                        uint32_t bc, yc, shp;
                        uint64_t ib, iy;
                        decode<false>(card, loc, bc, yc, shp, ib, iy);
                        score_one(bc, yc, ib, iy, shp, ~(key_l | ((c0 + loc) & 0xFFFFFF)));
                    }
                    __syncwarp();
                };
                // a warp covers 128 consecutive candidates per step, as two
                // halves of 64 (two per lane) whose loads are issued together;
                // the ring is drained after each half (it never holds more than
                // 31 + 64 entries)
                auto push = [&](const uint4 w, uint32_t c) {
                    const uint32_t s0 = (w.x >> 24) + (w.y >> 24), s1 = (w.z >> 24) + (w.w >> 24);
                    const bool q0 = s0 >= a.thr && c < ntile, q1 = s1 >= a.thr && c + 1 < ntile;  // thr = max(min_shp, 1)
                    const uint32_t b0 = __ballot_sync(0xFFFFFFFFu, q0), b1 = __ballot_sync(0xFFFFFFFFu, q1);
                    if ((b0 | b1) == 0) return;
                    const uint32_t lt = (1u << lane) - 1u;
                    const uint32_t r = qhead + qh + (uint32_t)(__popc(b0 & lt) + __popc(b1 & lt));
                    if (q0) wq[r & (kWQ - 1)] = (uint16_t)c;
                    if (q1) wq[(r + (q0 ? 1u : 0u)) & (kWQ - 1)] = (uint16_t)(c + 1);
                    qh += (uint32_t)(__popc(b0) + __popc(b1));
                    while (qh >= 32)
                    {
                        pop_score(32);
                        qhead += 32;
                        qh -= 32;
                    }
                };
                const uint32_t first = 4 * (tid - (uint32_t)lane), step = 4 * nthr;
                const uint32_t thr4 = min(a.thr, 255u) * 0x01010101u;
                const bool thr7 = a.thr <= 127u;
                for (uint32_t base = first; base < ntile; base += step)
                {
                    // words past ntile are zero up to the tile's end (the clear
                    // leaves every word past the next job's end zero) and past
                    // it belong to the queue: a window's last step is masked
                    const uint32_t ca = base + 2 * (uint32_t)lane, cb = ca + 64;
                    const uint4 wa = c4[ca >> 1];
                    const uint4 wb = c4[cb >> 1];
                    // the four candidates' counts (the top bytes of their b and y
                    // words) summed and compared as bytes: candidates ca, ca + 1,
                    // cb, cb + 1 in bytes 0..3 (each count < 128, so no carry)
                    const uint32_t bw = __byte_perm(__byte_perm(wa.x, wa.z, 0x0073u), __byte_perm(wb.x, wb.z, 0x0073u),
                                                    0x5410u);
                    const uint32_t yw = __byte_perm(__byte_perm(wa.y, wa.w, 0x0073u), __byte_perm(wb.y, wb.w, 0x0073u),
                                                    0x5410u);
                    // (a plain add: each sum is below 256). Byte k's top bit of m:
                    // its sum reaches thr; for thr <= 127, (sum | 0x80) - thr
                    // keeps the top bit exactly when sum >= thr, with no borrow
                    // between bytes, and a sum of 128 or more has it already
                    const uint32_t sw = bw + yw;
                    uint32_t m = thr7 ? (((sw | 0x80808080u) - thr4) | sw) & 0x80808080u
                                      : (__vcmpgeu4(sw, thr4) & 0x01010101u) << 7;
                    if (base + 128u > ntile)  // warp-uniform
                        m &= (ca < ntile ? 0x80u : 0u) | (ca + 1u < ntile ? 0x8000u : 0u) |
                             (cb < ntile ? 0x800000u : 0u) | (cb + 1u < ntile ? 0x80000000u : 0u);
                    // this lane's place in the warp's ring: from the warp's
                    // append counter (T.wtail = qhead + qh; lanes in any order)
                    const uint32_t n4 = __popc(m);
                    const uint32_t tot = __reduce_add_sync(0xFFFFFFFFu, n4);
                    if (tot == 0) continue;
                    if (qh + tot <= kWQ)
                    {
                        uint32_t r = n4 ? atomicAdd(&T.wtail[wid], n4) : 0u;
                        while (m)
                        {
                            const int k = (__ffs(m) - 1) >> 3;
                            m &= m - 1;
                            wq[r & (kWQ - 1)] = (uint16_t)((k < 2 ? ca : cb) + (uint32_t)(k & 1));
                            r++;
                        }
                        qh += tot;
                        while (qh >= 32)
                        {
                            pop_score(32);
                            qhead += 32;
                            qh -= 32;
                        }
                    }
                    else
                    {
                        // the ring would overflow: the two halves one after the other
                        push(wa, ca);
                        push(wb, cb);
                        __syncwarp();
                        if (lane == 0) T.wtail[wid] = qhead + qh;
                        __syncwarp();
                    }
                }
                if (qh) pop_score(qh);
                // the next job's candidates and their classes (its scorecard start)
                const uint32_t nn = nj.l != kNoJob ? nj.c1 - nj.c0 : 0u;
                const uint8_t *ncls = nn ? a.len[nj.l].cls + nj.c0 : nullptr;
                // the warp's own words, now read: the next job's start there,
                // four consecutive candidates per lane (b word zero, y word
                // its class's adds; zero past the next job's end)
                uint4 *z4 = reinterpret_cast<uint4 *>(card);
                const uint32_t lim = max(ntile, nn);
                const bool al4 = (nj.c0 & 3u) == 0u;  // class bytes readable as one word (warp-uniform)
                for (uint32_t base = first; base < lim; base += step)
                {
                    const uint32_t c = base + 4 * (uint32_t)lane;
                    uint32_t k4 = kClassNone * 0x01010101u;
                    if (c < nn)
                    {
                        if (al4) k4 = __ldg(reinterpret_cast<const uint32_t *>(ncls + c));
                        else
                            k4 = (uint32_t)__ldg(ncls + c) | ((uint32_t)__ldg(ncls + c + 1) << 8) |
                                 ((uint32_t)__ldg(ncls + c + 2) << 16) | ((uint32_t)__ldg(ncls + c + 3) << 24);
                        if (c + 4 > nn)
                        {
                            const uint32_t keep = (1u << (8 * (nn - c))) - 1u;  // bytes of candidates < nn
                            k4 = (k4 & keep) | (kClassNone * 0x01010101u & ~keep);
                        }
                    }
                    const uint32_t y0 = T.upk[k4 & 0xFFu], y1 = T.upk[(k4 >> 8) & 0xFFu];
                    const uint32_t y2 = T.upk[(k4 >> 16) & 0xFFu], y3 = T.upk[k4 >> 24];
                    if (c < lim)  // words from lim on are zero already (and past the tile not its own)
                    {
                        z4[c >> 1] = make_uint4(0u, y0, 0u, y1);
                        z4[(c >> 1) + 1] = make_uint4(0u, y2, 0u, y3);
                    }
                    npass += (y0 >> 24) + (y1 >> 24) + (y2 >> 24) + (y3 >> 24);
                }
            }
            else
            {
                // wide words: one candidate per thread, every one checked, then
                // set to the next job's start (y word: class adds; zero past its end)
                const uint32_t nn = nj.l != kNoJob ? nj.c1 - nj.c0 : 0u;
                const uint8_t *ncls = nn ? a.len[nj.l].cls + nj.c0 : nullptr;
                const uint32_t lim = max(ntile, nn);
                for (uint32_t c = tid; c < lim; c += nthr)
                {
                    if (c < ntile)
                    {
                        uint32_t bc, yc, shp;
                        uint64_t ib, iy;
                        decode<WIDE>(card, c, bc, yc, shp, ib, iy);
                        if (shp >= a.min_shp && shp != 0)
                            score_one(bc, yc, ib, iy, shp, ~(key_l | ((c0 + c) & 0xFFFFFF)));
                    }
                    W wy = 0;
                    if (c < nn)
                    {
                        wy = ucls[__ldg(ncls + c)];
                        npass += (uint32_t)(wy >> 40);
                    }
                    card[2 * c] = 0;
                    card[2 * c + 1] = wy;
                }
            }
            {
                my_cps = __reduce_add_sync(0xFFFFFFFFu, my_cps);
                my_fl = __reduce_or_sync(0xFFFFFFFFu, my_fl);
                if (lane == 0)
                {
                    if (my_cps) atomicAdd(&T.cpsms, my_cps);
                    if (my_fl) atomicOr(&T.flags, my_fl);
                }
                if (a.phase && my_exact) atomicAdd(&T.cnt[3], (unsigned long long)my_exact);
                if (a.phase && tid == 0) T.cnt[0] += 1;
            }
            HC_PHASE(2);
            if (tid == 0) T.pnext = 0;
            __syncthreads();
            HC_PHASE(3);
            jb = nj;
        }
        // ---- candidates whose sign or bin the float estimate left open ----
        if (!WIDE)
        {
            const uint32_t nd = min(T.ndefer, a.defer_cap);
            uint32_t cps = 0, fl = 0, nex = 0;
            for (uint32_t i = tid; i < nd; i += nthr)
            {
                uint32_t bc, yc, shp;
                uint64_t ib, iy;
                const uint2 w = defer[i];
                decode_packed(w.x, w.y, bc, yc, shp, ib, iy);
                nex++;
                const float h = exact_h(a.qc, bc, yc, ib, iy);
                if (!(h > 0.0f)) continue;
                int bin = hist_bin(h);
                cps++;
                if (bc >= (uint32_t)kRefMaxShp || yc >= (uint32_t)kRefMaxShp) fl |= HC_FLAG_LGFACT_OOB;
                if (bin >= HC_HIST_BINS || bin < 0) { fl |= HC_FLAG_HIST_OOB; bin = bin < 0 ? 0 : HC_HIST_BINS - 1; }
                hist_add(bin);
            }
            cps = __reduce_add_sync(0xFFFFFFFFu, cps);
            fl = __reduce_or_sync(0xFFFFFFFFu, fl);
            if (lane == 0)
            {
                if (cps) atomicAdd(&T.cpsms, cps);
                if (fl) atomicOr(&T.flags, fl);
            }
            if (a.phase && nex) atomicAdd(&T.cnt[3], (unsigned long long)nex);
        }
        // postings visited: those of entries inside the window
        npass = __reduce_add_sync(0xFFFFFFFFu, npass);
        if (lane == 0 && npass) atomicAdd(&T.bytes, 4ull * npass);
        // the top hit's shared ions come from the thread that found it
        if (my_best != 0 && my_best == T.best) T.best_shp = my_shp;
        __syncthreads();
        HC_PHASE(5);
        // ---- write the spectrum's results ----
        if (!WIDE && T.overflow)
        {
            if (tid == 0)
            {
                const uint32_t wi = atomicAdd(a.nwide, 1u);
                a.wide_list[wi] = s;
            }
            continue;
        }
        for (int i = tid; i < kHistSm; i += nthr) a.hist[(size_t)s * HC_HIST_BINS + i] = T.u.run.hist[i];
        if (tid == 0)
        {
            hc_result r;
            r.cpsms = T.cpsms;
            r.flags = T.flags;
            r.post_bytes = T.bytes;
            if (T.cpsms > 0 && T.best != 0)
            {
                const uint32_t tie = ~(uint32_t)(T.best & 0xFFFFFFFFu);
                r.idxoffset = (int32_t)(tie >> 24);
                r.psid = (int32_t)(tie & 0xFFFFFF);
                r.hyperscore = __uint_as_float((uint32_t)(T.best >> 32));
                r.sharedions = (uint16_t)T.best_shp;
                r.totalions = (uint16_t)a.lens[r.idxoffset].speclen;
            }
            else
            {
                r.idxoffset = -1;
                r.psid = -1;
                r.hyperscore = 0.0f;
                r.sharedions = 0;
                r.totalions = 0;
            }
            r.mu = r.beta = r.minhyp = r.nexthyp = r.maxhyp = 0;
            r.reported = 0;
            r.evalue = 0.0;
            a.out[s] = r;
        }
    }
    if (a.phase && tid == 0)
    {
        for (int k = 0; k < kPhases; k++) atomicAdd(&a.phase[k], T.ph[k]);
        for (int k = 0; k < 4; k++) atomicAdd(&a.phase[kPhases + k], T.cnt[k]);
    }
}

// ---- windows: DSLIM_BinarySearch (dslim_query.cpp:854-994) -----------------
__device__ int find_min(const float *__restrict__ m, float pm, int mn, int mx)
{
    for (;;)
    {
        int half = (mn + mx) / 2;
        if (mx - mn < 20)
        {
            int cur = mn;
            while (__ldg(m + cur) < pm) cur++;
            return cur;
        }
        const float v = __ldg(m + half);
        if (pm > v) { mn = half; continue; }
        if (pm < v) { mx = half; continue; }
        while (half >= 0 && pm == __ldg(m + half)) half--;
        return half + 1;
    }
}

__device__ int find_max(const float *__restrict__ m, int n, float pm, int mn, int mx)
{
    for (;;)
    {
        int half = (mn + mx) / 2;
        if (mx - mn < 20)
        {
            int cur = mx;
            while (__ldg(m + cur) > pm) cur--;
            return cur;
        }
        const float v = __ldg(m + half);
        if (pm > v) { mn = half; continue; }
        if (pm < v) { mx = half; continue; }
        half++;
        while (half < n && pm == __ldg(m + half)) half++;
        return half - 1;
    }
}

__global__ void k_windows(const LenDev *__restrict__ lens, uint32_t nlen, const float *__restrict__ prec,
                          const double *__restrict__ dMs, double dM0, uint32_t nspec, int2 *__restrict__ win)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (uint64_t)nspec * nlen) return;
    const uint32_t s = (uint32_t)(g / nlen), l = (uint32_t)(g % nlen);
    const double dM = dMs ? dMs[s] : dM0;
    const float pm = prec[s];
    // float pmass1 = precmass - params.dM: double difference rounded to float
    const float pm1 = __double2float_rn(__dadd_rn((double)pm, -dM));
    const float pm2 = __double2float_rn(__dadd_rn((double)pm, dM));
    const int n = (int)lens[l].n;
    const float *m = lens[l].mass;
    int2 r = make_int2(1, 0);
    if (n > 0 && !(dM < 0.0))
    {
        int mn = 0, mx = n - 1, lo, hi;
        bool ok = true;
        if (pm1 < __ldg(m + mn)) lo = mn;
        else if (pm1 > __ldg(m + mx)) ok = false;
        else lo = find_min(m, pm1, mn, mx);
        if (ok)
        {
            if (pm2 > __ldg(m + mx)) hi = mx;
            else if (pm2 < __ldg(m + mn)) ok = false;
            else hi = find_max(m, n, pm2, mn, mx);
        }
        if (ok && __ldg(m + hi) <= pm2 && __ldg(m + lo) >= pm1 && hi >= lo) r = make_int2(lo, hi);
    }
    win[g] = r;
}

// ---- tail fit + e-value ------------------------------------------------------
constexpr int kTfWarps = 4;

// expeRT::ModelTailFit (expeRT.cpp:572-718) and e(x) (dslim_query.cpp:773-799)
// of spectrum s, by one warp. Elementwise steps run across lanes; the sums
// whose rounding depends on order (ybar, top, bot of LinearFit) run on lane 0
// in the reference's order. Cumulative sums are exact integers either way.
// sx: the warp's HC_HIST_BINS + 2 doubles of shared memory.
__device__ void tailfit_one(uint32_t s, hc_result *__restrict__ out, const uint32_t *__restrict__ hist,
                            uint32_t min_cpsm, double expect_max, int32_t *__restrict__ fitstart, double *sx,
                            int lane)
{
    hc_result r = out[s];
    r.mu = r.beta = r.minhyp = r.nexthyp = r.maxhyp = 0;
    r.evalue = 0.0;
    r.reported = 0;
    if (r.cpsms < min_cpsm || r.cpsms == 0)
    {
        if (lane == 0)
        {
            out[s] = r;
            fitstart[s] = -1;
        }
        return;
    }
    int fit_first = -1;  // first regression bin (the learned tail's third target)
    const uint32_t *yy = hist + (size_t)s * HC_HIST_BINS;
    const int hyp = hist_bin(r.hyperscore);  // maxhypscore (dslim_query.cpp:778)
    const int cps = (int)r.cpsms;
    // expeRT.cpp:590-598: end1 = last bin below hyp holding >= 1, stt1 = first
    int stt1, end1;
    const int n = tail_bins(yy, hyp, HC_HIST_BINS, lane, stt1, end1);
    double mu_t = 0.0, beta_t = 0.0;
    uint32_t fl = 0;
    if (n == 0)
    {
        fl |= HC_FLAG_TAILFIT_EMPTY;  // LinearFit of 0 points: 0/0
        mu_t = beta_t = __longlong_as_double(0x7FF8000000000000ll);
    }
    else
    {
        // s(x) = -(cumsum/cpsms + -1), values > 1 -> 0.999 (expeRT.cpp:625-636)
        unsigned long long carry = 0;
        for (int i0 = 0; i0 < n; i0 += 32)
        {
            const int i = i0 + lane;
            unsigned long long v = (i < n) ? yy[stt1 + i] : 0ull;
            for (int o = 1; o < 32; o <<= 1)
            {
                const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, v, o);
                if (lane >= o) v += t;
            }
            if (i < n)
            {
                double d = __ddiv_rn((double)(carry + v), (double)cps);
                d = -__dadd_rn(d, -1.0);
                if (d > 1.0) d = 0.999;
                sx[i + 1] = d;
            }
            carry += __shfl_sync(0xFFFFFFFFu, v, 31);
        }
        if (lane == 0) sx[0] = 0.0;
        __syncwarp();
        // values <= 0 take the last value >= 1e-4 (expeRT.cpp:639-640), then log10
        int repl = n - 1;
        for (int q0 = n - 1; q0 >= 0; q0 -= 32)
        {
            const int q = q0 - lane;
            const uint32_t b = __ballot_sync(0xFFFFFFFFu, q >= 0 && sx[q + 1] >= 1e-4);
            if (b) { repl = q0 - (__ffs(b) - 1); break; }
        }
        const double rv = sx[repl + 1];
        __syncwarp();
        for (int i = lane; i < n; i += 32)
        {
            double v = sx[i + 1];
            if (v <= 0.0) v = rv;
            sx[i + 1] = log10(v);
        }
        __syncwarp();
        // regression window (expeRT.cpp:646-684)
        int mark = 0, mark2 = n - 1;
        const double hgt = __dadd_rn(sx[n], -sx[1]);
        if (n >= 3)
        {
            const double t1 = __dadd_rn(sx[1], __dmul_rn(hgt, 0.22));
            int lm = 0;
            for (int q0 = 0; q0 < n; q0 += 32)
            {
                const int q = q0 + lane;
                const uint32_t b = __ballot_sync(0xFFFFFFFFu, q < n && sx[q + 1] <= t1);
                if (b) { lm = q0 + __ffs(b) - 1; break; }
            }
            mark = lm - 1;
            if (n > 3)
            {
                const double t2 = __dadd_rn(sx[1], __dmul_rn(hgt, 0.87));
                for (int q0 = n - 1; q0 >= 0; q0 -= 32)
                {
                    const int q = q0 - lane;
                    const uint32_t b = __ballot_sync(0xFFFFFFFFu, q >= 0 && sx[q + 1] >= t2);
                    if (b) { mark2 = q0 - (__ffs(b) - 1); break; }
                }
            }
            if (mark >= mark2) mark = mark2 - 1;
        }
        if (mark < 0) fl |= HC_FLAG_TAILFIT_OOB;  // reads element -1 (sx[0] = +0.0)
        fit_first = stt1 + mark;
        const int m = mark2 - mark + 1;
        const double *y = sx + 1 + mark;
        // LinearFit (expeRT.cpp:1297-1345) on lane 0, in the reference's order
        if (lane == 0)
        {
            if (m == 1)
            {
                mu_t = 0.0;
                beta_t = y[0];
            }
            else
            {
                double xbar = 0.0, ybar = 0.0, top = 0.0, bot = 0.0;
                for (int i = 0; i < m; i++)
                {
                    xbar = __dadd_rn(xbar, (double)(stt1 + mark + i));
                    ybar = __dadd_rn(ybar, y[i]);
                }
                xbar = __ddiv_rn(xbar, (double)m);
                ybar = __ddiv_rn(ybar, (double)m);
                for (int i = 0; i < m; i++)
                {
                    const double dx = __dadd_rn((double)(stt1 + mark + i), -xbar);
                    top = __dadd_rn(top, __dmul_rn(dx, __dadd_rn(y[i], -ybar)));
                    bot = __dadd_rn(bot, __dmul_rn(dx, dx));
                }
                mu_t = __ddiv_rn(top, bot);
                beta_t = __dadd_rn(ybar, -__dmul_rn(mu_t, xbar));
            }
        }
    }
    if (lane == 0)
    {
        fitstart[s] = fit_first;
        r.flags |= fl;
        r.mu = x86_d2i(__dmul_rn(mu_t, 1e6));
        r.beta = x86_d2i(__dmul_rn(beta_t, 1e6));
        r.minhyp = stt1;
        r.nexthyp = end1;
        r.maxhyp = hyp;
        // e(x) = 10^(w*maxhyp + b) * cpsms (dslim_query.cpp:786-799)
        const double wv = __ddiv_rn((double)r.mu, 1e6), bv = __ddiv_rn((double)r.beta, 1e6);
        const double lgs = __dadd_rn(__dmul_rn(wv, (double)hyp), bv);
        double e = pow(10.0, lgs);
        e = __dmul_rn(e, (double)r.cpsms);
        r.evalue = e;
        r.reported = e < expect_max ? 1u : 0u;
        out[s] = r;
    }
}

// One warp per spectrum: every spectrum of [0, nspec), or those of `list`
// (its length *nlist read on the device) when a list is given.
__global__ void __launch_bounds__(kTfWarps * 32) k_tailfit(hc_result *__restrict__ out,
                                                          const uint32_t *__restrict__ hist,
                                                          uint32_t nspec, uint32_t min_cpsm,
                                                          double expect_max, int32_t *__restrict__ fitstart,
                                                          const uint32_t *__restrict__ list,
                                                          const uint32_t *__restrict__ nlist)
{
    __shared__ double sxs[kTfWarps][HC_HIST_BINS + 2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *sx = sxs[warp];  // sx[0] stands for index -1; element i is sx[i + 1]
    const uint32_t cnt = list ? min(*nlist, nspec) : nspec;
    for (uint32_t w = blockIdx.x * kTfWarps + warp; w < cnt; w += gridDim.x * kTfWarps)
    {
        tailfit_one(list ? list[w] : w, out, hist, min_cpsm, expect_max, fitstart, sx, lane);
        __syncwarp();
    }
}

// ---- longest-first order for the batched schedule --------------------------
// cost class of a spectrum = bit length of its total window size (candidates)
constexpr int kCostClasses = 64;

__global__ void k_cost(const int2 *__restrict__ win, uint32_t nspec, uint32_t nlen, uint32_t *__restrict__ cls,
                       uint32_t *__restrict__ cnt)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    unsigned long long c = 0;
    for (uint32_t l = 0; l < nlen; l++)
    {
        const int2 w = win[(size_t)s * nlen + l];
        if (w.y >= w.x) c += (unsigned long long)(w.y - w.x + 1);
    }
    const uint32_t k = c ? 64u - (uint32_t)__clzll(c) : 0u;
    cls[s] = k;
    atomicAdd(&cnt[k], 1u);
}

// split (optional): the number of spectra whose cost class exceeds
// split_class, i.e. whose windows hold 2^split_class candidates or more in all
// (they come first in the order)
__global__ void k_order(const uint32_t *__restrict__ cls, uint32_t nspec, const uint32_t *__restrict__ cnt,
                        uint32_t *__restrict__ cursor, uint32_t *__restrict__ order, uint32_t split_class,
                        uint32_t *__restrict__ split)
{
    __shared__ uint32_t off[kCostClasses];
    if (threadIdx.x == 0)
    {
        uint32_t run = 0;
        for (int k = kCostClasses - 1; k >= 0; k--)
        {
            off[k] = run;
            run += cnt[k];
        }
        if (split && blockIdx.x == 0) *split = off[split_class];
    }
    __syncthreads();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const uint32_t k = cls[s];
    order[off[k] + atomicAdd(&cursor[k], 1u)] = s;
}

}  // namespace

size_t search_smem(uint32_t tile, uint32_t dF, bool wide, uint32_t threads)
{
    return smem_layout(tile, dF, wide, threads / 32).total;
}

template <class T>
static int grow(hc_ctx *ctx, T **p, size_t *cap, size_t need);

// the largest tile (a multiple of kRowG) whose whole layout fits in `budget` bytes
static uint32_t fit_tile(size_t budget, uint32_t dF, uint32_t threads)
{
    uint32_t t = (uint32_t)std::min<size_t>(budget / 8, 32768) / kRowG * kRowG;  // ring entries are 16-bit
    while (t > kRowG && smem_layout(t, dF, false, threads / 32).total > budget) t -= kRowG;
    return t < kRowG ? kRowG : t;
}

// Stage timing event; inside a stream capture it becomes an external event
// record node, so a replayed graph still times its stages.
cudaError_t record_stage(hc_ctx *ctx, int i, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ctx->ev[i], st, cudaEventRecordExternal)
                                               : cudaEventRecord(ctx->ev[i], st);
}

// Shared memory the resident CTAs take at most when a tile is picked, so that
// the SM keeps 60 KB of its 256 KB as L1 (the next configuration down keeps
// 28 KB): the search reads its jobs' class codes and row-table words through
// L1, and with 28 KB it runs 9-10 % slower at the same tile.
constexpr size_t kSmemKeepL1 = 196 * 1024;

uint32_t max_tile(const hc_ctx *ctx, uint32_t dF, uint32_t threads)
{
    return max_tile_for(ctx, dF, 1, threads);
}

uint32_t max_tile_for(const hc_ctx *ctx, uint32_t dF, uint32_t ctas_per_sm, uint32_t threads)
{
    if (ctas_per_sm < 1) ctas_per_sm = 1;
    // the SM's shared memory is split; each CTA also keeps a reserve for the system
    const size_t full = std::min(ctx->smem_optin, ctx->smem_sm / ctas_per_sm - ctx->smem_reserved);
    const size_t keep = std::min(full, kSmemKeepL1 / ctas_per_sm - ctx->smem_reserved);
    for (const size_t per : {keep, full})
    {
        const uint32_t t = fit_tile(per, dF, threads);
        if (smem_layout(t, dF, false, threads / 32).total <= per) return t;
    }
    return 0u;
}

int prepare_query(hc_ctx *ctx, uint32_t nspec)
{
    int rc = sync_lengths(ctx);
    if (rc) return rc;
    const uint32_t nlen = (uint32_t)ctx->lens.size();
    QueryScratch &q = ctx->qs;
    if ((rc = grow(ctx, &q.d_win, &q.win_cap, (size_t)nspec * nlen))) return rc;
    if ((rc = grow(ctx, &q.d_wide, &q.wide_cap, (size_t)nspec + 4))) return rc;
    if ((rc = grow(ctx, &q.d_order, &q.order_cap, 2 * (size_t)nspec))) return rc;
    if ((rc = grow(ctx, &q.d_fitstart, &q.fit_cap, (size_t)nspec))) return rc;
    if (!q.d_work) HC_CUDA(ctx, cudaMalloc((void **)&q.d_work, 4 * kWorkWords));
    return HC_SUCCESS;
}

namespace {

template <bool WIDE, int G>
int launch_g(hc_ctx *ctx, const SearchArgs &a, int grid, uint32_t threads, size_t smem, cudaStream_t st)
{
    if (G >= 4 && threads > 512) threads = 512;
    HC_CUDA(ctx, cudaFuncSetAttribute(k_search<WIDE, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_search<WIDE, G><<<grid, threads, smem, st>>>(a);
    HC_CUDA(ctx, cudaGetLastError());
    return HC_SUCCESS;
}

template <bool WIDE>
int launch_search(hc_ctx *ctx, const SearchArgs &a, int grid, uint32_t threads, size_t smem, uint32_t g,
                  cudaStream_t st)
{
    switch (g)
    {
    case 1: return launch_g<WIDE, 1>(ctx, a, grid, threads, smem, st);
    case 2: return launch_g<WIDE, 2>(ctx, a, grid, threads, smem, st);
    case 8: return launch_g<WIDE, 8>(ctx, a, grid, threads, smem, st);
    default: return launch_g<WIDE, 4>(ctx, a, grid, threads, smem, st);
    }
}

}  // namespace

// the device record of one length
static void fill_lendev(const hc_ctx *ctx, const LenHost &lh, LenDev &d)
{
    std::memset(&d, 0, sizeof(d));
    d.L = lh.L;
    d.n = lh.built ? lh.n : 0;
    d.npep = lh.npep;
    d.speclen = 2 * ctx->p.maxz * (lh.L - 1);
    d.half = d.speclen / 2;
    division_magic(d.speclen, &d.magic, &d.msh);
    d.stride = lh.stride;
    d.mass = lh.d_mass;
    d.seqid = lh.d_seqid;
    d.sites = lh.d_sites;
    d.modnum = lh.d_modnum;
    d.seqs = lh.d_seqs;
    d.bA = lh.d_bA;
    d.qA = lh.d_qA;
    d.qp = lh.d_qp;
    d.qps = lh.d_qps;
    d.rows = lh.d_rows;
    d.cls = lh.d_cls;
}

// the length records the search kernel keeps in its parameters
static void fill_lens(const hc_ctx *ctx, SearchArgs &a)
{
    for (size_t i = 0; i < ctx->lens.size(); i++)
    {
        const LenHost &lh = ctx->lens[i];
        a.len[i] = LenS{lh.d_qps, lh.d_rows, lh.stride, lh.built ? lh.n : 0u, lh.d_cls};
    }
}

int sync_lengths(hc_ctx *ctx)
{
    if (!ctx->lens_dirty) return HC_SUCCESS;
    const uint32_t nlen = (uint32_t)ctx->lens.size();
    std::vector<LenDev> h(nlen);
    for (uint32_t i = 0; i < nlen; i++)
    {
        fill_lendev(ctx, ctx->lens[i], h[i]);
    }
    if (!ctx->d_lens) HC_CUDA(ctx, cudaMalloc((void **)&ctx->d_lens, sizeof(LenDev) * HC_MAX_LENGTHS));
    HC_CUDA(ctx, cudaMemcpy(ctx->d_lens, h.data(), sizeof(LenDev) * nlen, cudaMemcpyHostToDevice));
    ctx->lens_dirty = false;
    return HC_SUCCESS;
}

template <class T>
static int grow(hc_ctx *ctx, T **p, size_t *cap, size_t need)
{
    if (*cap >= need) return HC_SUCCESS;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    HC_CUDA(ctx, cudaMalloc((void **)p, sizeof(T) * need));
    *cap = need;
    return HC_SUCCESS;
}

// The packed search of a batch: with schedule 2 the longest-first order first,
// then one launch of the tuned shape or, when small windows have their own
// launch, two: the tuned shape takes the order up to the split point and
// 128-thread CTAs, kSmallCtas per SM, the rest (spectra that are mostly
// fixed per-job latency gain from more of them in flight per SM). Both read
// their range of the order on the device.
constexpr uint32_t kSmallThreads = 128, kSmallCtas = 6;

static int launch_packed(hc_ctx *ctx, SearchArgs &a, uint32_t sched, uint32_t nspec, uint32_t nlen, const int2 *win,
                         uint32_t *order, uint32_t *work, cudaStream_t st, int &launches, bool stages)
{
    const hc_tuning &t = ctx->tuning;
    const uint32_t small_tile = max_tile_for(ctx, a.dF, kSmallCtas, kSmallThreads);
    const bool split = sched == 2 && t.small_log2 != 0 && small_tile >= kRowG;
    a.obase = a.olim = nullptr;
    if (sched == 2)
    {
        uint32_t *cls = order + nspec;
        k_cost<<<(nspec + 255) / 256, 256, 0, st>>>(win, nspec, nlen, cls, work + kWkCnt);
        k_order<<<(nspec + 255) / 256, 256, 0, st>>>(cls, nspec, work + kWkCnt, work + kWkCur, order,
                                                     split ? t.small_log2 : 0u, split ? work + kWkSplit : nullptr);
        HC_CUDA(ctx, cudaGetLastError());
        a.order = order;
        launches += 2;
        if (split) a.olim = work + kWkSplit;
    }
    // the search stage: the packed launches
    if (stages) HC_CUDA(ctx, record_stage(ctx, 1, st));
    const size_t smem = search_smem(a.tile, a.dF, false, t.threads);
    const int grid = sched == 1 ? (int)nspec : ctx->sm_count * (int)t.ctas_per_sm;
    int rc = launch_search<false>(ctx, a, grid, t.threads, smem, t.pairs_per_warp, st);
    if (rc || !split) return rc;
    SearchArgs s = a;
    s.obase = work + kWkSplit;
    s.olim = nullptr;
    s.work = work + kWkSmall;
    s.tile = small_tile;
    s.always_return = 1;
    launches++;
    return launch_search<false>(ctx, s, ctx->sm_count * (int)kSmallCtas, kSmallThreads,
                                search_smem(small_tile, s.dF, false, kSmallThreads), 2, st);
}

int query_device(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_int,
                 const float *d_prec, const double *d_dM, uint32_t nspec, uint32_t npeaks,
                 hc_result *d_out, uint32_t *d_hist, cudaStream_t st, bool tailfit)
{
    (void)npeaks;
    int rc = sync_lengths(ctx);
    if (rc) return rc;
    ctx->last_launches = 0;
    ctx->last_learned = !tailfit;
    if (nspec == 0) return HC_SUCCESS;
    const uint32_t nlen = (uint32_t)ctx->lens.size();
    QueryScratch &q = ctx->qs;
    if ((rc = grow(ctx, &q.d_win, &q.win_cap, (size_t)nspec * nlen))) return rc;
    if ((rc = grow(ctx, &q.d_wide, &q.wide_cap, (size_t)nspec + 4))) return rc;
    const uint32_t sched = ctx->tuning.schedule;
    if (sched == 2 && (rc = grow(ctx, &q.d_order, &q.order_cap, 2 * (size_t)nspec))) return rc;
    if ((rc = grow(ctx, &q.d_fitstart, &q.fit_cap, (size_t)nspec))) return rc;
    if (!q.d_work) HC_CUDA(ctx, cudaMalloc((void **)&q.d_work, 4 * kWorkWords));
    q.d_nwide = q.d_work + kWkNwide;
    HC_CUDA(ctx, cudaMemsetAsync(q.d_work, 0, 4 * kWorkWords, st));

    const uint64_t nw = (uint64_t)nspec * nlen;
    if (ctx->profiling) HC_CUDA(ctx, record_stage(ctx, 0, st));
    k_windows<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(ctx->d_lens, nlen, d_prec, d_dM, ctx->p.dM,
                                                            nspec, q.d_win);
    HC_CUDA(ctx, cudaGetLastError());

    SearchArgs a{};
    a.lens = ctx->d_lens;
    fill_lens(ctx, a);
    a.nlen = nlen;
    a.qc = ctx->d_qconst;
    a.idx = d_idx;
    a.moz = d_moz;
    a.inten = d_int;
    a.prec = d_prec;
    a.win = q.d_win;
    a.nspec = nspec;
    a.dF = ctx->p.dF;
    a.min_shp = ctx->p.min_shp;
    a.thr = ctx->p.min_shp > 0 ? ctx->p.min_shp : 1;
    a.maxbin = ctx->p.max_mass * ctx->p.scale;
    a.out = d_out;
    a.hist = d_hist;
    a.wide_list = q.d_wide;
    a.nwide = q.d_nwide;
    a.work = q.d_work;
    a.tile = ctx->tuning.tile;
    a.defer_cap = ctx->tuning.defer_cap;
    a.persistent = sched != 1;
    a.maxz = ctx->p.maxz;
    a.classes = ctx->d_classes;
    a.phase = ctx->d_phase;
    int launches = 4;
    int rc2 = launch_packed(ctx, a, sched, nspec, nlen, q.d_win, q.d_order, q.d_work, st, launches, ctx->profiling);
    if (rc2) return rc2;
    if (ctx->profiling) HC_CUDA(ctx, record_stage(ctx, 2, st));
    // spectra whose packed scorecard could overflow are redone wide; the
    // list length is read on the device (no host synchronisation)
    SearchArgs b = a;
    b.persistent = 1;
    b.phase = nullptr;
    b.order = nullptr;
    b.only = q.d_wide;
    b.nonly_dev = q.d_nwide;
    b.work = q.d_work + kWkWide;
    b.obase = b.olim = nullptr;
    b.tile = std::max(kRowG, ctx->tuning.tile / 2 / kRowG * kRowG);  // same shared memory, 16-byte words
    const size_t smem2 = search_smem(b.tile, b.dF, true, ctx->tuning.threads);
    rc2 = launch_search<true>(ctx, b, ctx->sm_count, ctx->tuning.threads, smem2, 2, st);
    if (rc2) return rc2;
    if (ctx->profiling) HC_CUDA(ctx, record_stage(ctx, 3, st));
    if (tailfit)
    {
        k_tailfit<<<(nspec + kTfWarps - 1) / kTfWarps, kTfWarps * 32, 0, st>>>(
            d_out, d_hist, nspec, ctx->p.min_cpsm, ctx->p.expect_max, q.d_fitstart, nullptr, nullptr);
        HC_CUDA(ctx, cudaGetLastError());
    }
    else
        launches--;
    if (ctx->profiling) HC_CUDA(ctx, record_stage(ctx, 4, st));
    ctx->last_launches = launches;
    return HC_SUCCESS;
}

namespace {

// The length table of one query, passed by value as a kernel parameter
// (7 KB, inside the 32 KB parameter space), so that writing it to device
// scratch needs neither a host copy nor a host buffer that must outlive the call.
struct LenTable
{
    LenDev l[HC_MAX_LENGTHS];
};

__global__ void k_put_lens(const LenTable t, uint32_t nlen, LenDev *__restrict__ dst)
{
    if (threadIdx.x < nlen) dst[threadIdx.x] = t.l[threadIdx.x];
}

template <class F>
cudaError_t load_one(F *f)
{
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, f);
}

}  // namespace

// Loads every kernel launch_query_scratch can launch into the current
// context. With lazy module loading (the default) a kernel's code is loaded,
// and device memory allocated for it, at its first launch; asking for its
// attributes loads it now instead.
int preload_query_kernels(hc_ctx *ctx)
{
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(load_one(k_put_lens));
    chk(load_one(k_windows));
    chk(load_one(k_cost));
    chk(load_one(k_order));
    chk(load_one(k_tailfit));
    chk(load_one(k_search<false, 1>));
    chk(load_one(k_search<false, 2>));
    chk(load_one(k_search<false, 4>));
    chk(load_one(k_search<false, 8>));
    chk(load_one(k_search<true, 2>));
    HC_CUDA(ctx, e);
    return HC_SUCCESS;
}

// The expeRT tail fit of the spectra in `list` (its length *d_nlist on the
// device, at most nmax): the fallback of the learned tail.
int tailfit_list(hc_ctx *ctx, hc_result *d_out, const uint32_t *d_hist, const uint32_t *list,
                 const uint32_t *d_nlist, uint32_t nmax, cudaStream_t st)
{
    if (nmax == 0) return HC_SUCCESS;
    QueryScratch &q = ctx->qs;
    int rc = grow(ctx, &q.d_fitstart, &q.fit_cap, (size_t)nmax);
    if (rc) return rc;
    const uint32_t blocks = std::min<uint32_t>((nmax + kTfWarps - 1) / kTfWarps, (uint32_t)ctx->sm_count * 16);
    k_tailfit<<<blocks, kTfWarps * 32, 0, st>>>(d_out, d_hist, nmax, ctx->p.min_cpsm, ctx->p.expect_max,
                                                q.d_fitstart, list, d_nlist);
    HC_CUDA(ctx, cudaGetLastError());
    return HC_SUCCESS;
}

// The query pipeline of query_device with every scratch buffer supplied by
// the caller (used by the allocation-free entry point): the length table is
// written into s.lens by a kernel that takes it as a parameter, nothing is
// allocated and the host does not wait.
int launch_query_scratch(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_int,
                         const float *d_prec, const double *d_dM, uint32_t nspec, hc_result *d_out,
                         uint32_t *d_hist, const ScratchPtrs &s, cudaStream_t st)
{
    const uint32_t nlen = (uint32_t)ctx->lens.size();
    LenTable t;
    std::memset(&t, 0, sizeof(t));
    for (uint32_t i = 0; i < nlen; i++)
    {
        fill_lendev(ctx, ctx->lens[i], t.l[i]);
    }
    k_put_lens<<<1, HC_MAX_LENGTHS, 0, st>>>(t, nlen, s.lens);
    HC_CUDA(ctx, cudaGetLastError());
    ctx->last_launches = 0;
    if (nspec == 0) return HC_SUCCESS;
    uint32_t *nwide = s.work + kWkNwide;
    HC_CUDA(ctx, cudaMemsetAsync(s.work, 0, 4 * kWorkWords, st));
    const uint64_t nw = (uint64_t)nspec * nlen;
    k_windows<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(s.lens, nlen, d_prec, d_dM, ctx->p.dM, nspec, s.win);
    HC_CUDA(ctx, cudaGetLastError());
    SearchArgs a{};
    a.lens = s.lens;
    fill_lens(ctx, a);
    a.nlen = nlen;
    a.qc = ctx->d_qconst;
    a.idx = d_idx;
    a.moz = d_moz;
    a.inten = d_int;
    a.prec = d_prec;
    a.win = s.win;
    a.nspec = nspec;
    a.dF = ctx->p.dF;
    a.min_shp = ctx->p.min_shp;
    a.thr = ctx->p.min_shp > 0 ? ctx->p.min_shp : 1;
    a.maxbin = ctx->p.max_mass * ctx->p.scale;
    a.out = d_out;
    a.hist = d_hist;
    a.wide_list = s.wide;
    a.nwide = nwide;
    a.work = s.work;
    a.tile = ctx->tuning.tile;
    a.defer_cap = ctx->tuning.defer_cap;
    const uint32_t sched = ctx->tuning.schedule;
    a.persistent = sched != 1;
    a.maxz = ctx->p.maxz;
    a.classes = ctx->d_classes;
    int launches = 4;
    int rc = launch_packed(ctx, a, sched, nspec, nlen, s.win, s.order, s.work, st, launches, false);
    if (rc) return rc;
    SearchArgs b = a;
    b.persistent = 1;
    b.order = nullptr;
    b.only = s.wide;
    b.nonly_dev = nwide;
    b.work = s.work + kWkWide;
    b.obase = b.olim = nullptr;
    b.tile = std::max(kRowG, ctx->tuning.tile / 2 / kRowG * kRowG);  // same shared memory, 16-byte words
    rc = launch_search<true>(ctx, b, ctx->sm_count, ctx->tuning.threads, search_smem(b.tile, b.dF, true, ctx->tuning.threads), 2, st);
    if (rc) return rc;
    k_tailfit<<<(nspec + kTfWarps - 1) / kTfWarps, kTfWarps * 32, 0, st>>>(d_out, d_hist, nspec, ctx->p.min_cpsm,
                                                                            ctx->p.expect_max, s.fitstart, nullptr,
                                                                            nullptr);
    HC_CUDA(ctx, cudaGetLastError());
    ctx->last_launches = launches + 1;
    return HC_SUCCESS;
}

}  // namespace hc
