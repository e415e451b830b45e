// Internal declarations shared by the host API (hc_api.cpp) and the device
// code (hc_index.cu, hc_query.cu). Not installed; not part of the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "hicops_gb300.h"

namespace hc {

constexpr int kMaxZ = 8;           // fragment charges handled (the reference clamps maxz <= 5)
constexpr int kLgTable = 256;      // lgfact entries kept on the device (flagged past 80)
constexpr int kRefMaxShp = 81;     // MAX_SHDPEAKS + 1 (utils.h:110)
constexpr size_t kIaPad = 128;     // postings arrays are padded: the query reads aligned 16-byte groups
// Row table: for every bucket, the position of its first posting whose entry
// is >= k * kRowG, for k = 0 .. ceil(n / kRowG). Scorecard tiles are whole
// multiples of kRowG entries, so every interior tile boundary is a lookup.
constexpr uint32_t kRowG = 2048;
// Query postings: the same postings as the reference's iA (ids entry*speclen
// + ion, ascending inside each bucket), stored as
//   (entry << 3) | (isY << 2)
// which is the byte offset of the candidate's scorecard word (two 32-bit
// words per candidate, b then y) counted from entry 0: a tile starting at
// entry c0 finds a posting's word at x - (c0 << 3) with no further decoding.
// The ion of each posting (needed only to give the reference's ids back)
// sits in a parallel u16 array. Every bucket starts at a multiple of 4 words;
// the gaps hold kQpostPad, which lies past every tile.
constexpr uint32_t kQpostPad = 0xFFFFFFFFu;
constexpr uint32_t kQpEntryShift = 3;
constexpr uint32_t kQpMaxEntries = (1u << 29) - 2;  // entries of one length the encoding holds

// Entry classes. An entry's first y ion (y1), at every fragment charge, is
// fixed by a few facts about the entry: whether its mass is legal, whether it
// takes the mod-spectrum path (utils.cpp:378-505 when it carries mods), its
// last residue and the mod there. Those facts form a small "code"; entries
// with the same code share their y1 keys (a tryptic database has a few dozen
// codes, and y1 postings are about half of all the postings a search
// visits). Every code seen gets a class id with the class's keys; the search
// postings leave out the y1 postings of classed entries, and the search
// starts each candidate's y word with what its class's keys collect from the
// spectrum's peaks (the same count and intensity sum the left-out postings
// would have added). The index build checks every left-out posting against
// its class's key, so the code only has to be right for an entry to be
// classed, never for the results to be right. (The first b ion has as few
// codes, but its postings are a tenth of the total: classing it costs the
// search more per candidate than its postings do.)
constexpr uint32_t kMaxClasses = 127;   // class ids 0 .. 126
constexpr uint32_t kClassNone = 127;    // an entry without a class (adds nothing)
constexpr uint32_t kCodes = 1u << 10;   // codes: legal, path, last residue, mod at the last residue

// The class keys, per class and charge.
struct ClassKeys
{
    uint32_t n;         // classes
    uint32_t maxkey;    // the largest key of any class (peaks above it + dF cannot reach one)
    uint32_t key[kMaxClasses][kMaxZ];
};

// One peptide length's device-resident index. All arrays are device pointers.
struct LenDev
{
    uint32_t L, speclen, half, n;  // n = entries
    uint32_t npep;
    uint32_t magic, msh;           // floor(x / speclen) = umulhi(x, magic) >> msh, x < 2^31
    uint32_t stride;               // row-table entries per bucket: ceil(n / kRowG) + 1
    const float *mass;
    const uint32_t *seqid;
    const uint64_t *sites;
    const uint32_t *modnum;
    const uint8_t *seqs;
    const uint32_t *bA;
    const uint32_t *qA;            // bucket starts in qp (multiples of 4)
    const uint32_t *qp;            // query postings (see kQpostPad)
    const uint32_t *qps;           // search postings: qp without the y1 postings of classed entries
    const uint32_t *rows;          // row table over qps, [bucket][k] with `stride` entries per bucket
    const uint8_t *cls;            // per entry: its class (kClassNone: none)
};

// Integer ion-key tables, derived on the host with the reference's double
// arithmetic (utils.cpp:231-276 and 378-505; see hc_host.cpp).
struct IonTables
{
    uint32_t bf[26][kMaxZ];   // (uint)((GETAA(a, z+1) * scale) / (z+1))
    uint32_t yf[26][kMaxZ];   // (uint)(((GETAA(a, z+1) + H2O) * scale) / (z+1))
    uint32_t inc[26][kMaxZ];  // (uint)((GETAA(a, 0) * scale) / (z+1))
    uint32_t bfm[26][kMaxZ];  // (uint)(GETAA(a, z+1) * scale)          (mod spectra)
    uint32_t yfm[26][kMaxZ];  // (uint)((GETAA(a, z+1) + H2O) * scale)  (mod spectra)
    uint32_t incm[26];        // (uint)(GETAA(a, 0) * scale)             (mod spectra)
    uint32_t mod_mass[16];
    uint32_t maxz, scale, min_mass, max_mass;
};

constexpr uint32_t kLog10Tab = 1u << 24;  // log10(n) for every n the packed sums can reach

struct QueryConst
{
    double lgfact[kLgTable];   // log10(n!) exactly as utils.h:115-131 builds it
    float lgfact_f[kLgTable];  // the same, rounded to float (fast path)
    const double *log10_tab;   // device table: log10_tab[n] = log10(n), n < kLog10Tab (host libm values)
};

// Host-side record of one length.
struct LenHost
{
    uint32_t L = 0, npep = 0, n = 0;
    uint64_t npost = 0;
    float *d_mass = nullptr;
    uint32_t *d_seqid = nullptr;
    uint64_t *d_sites = nullptr;
    uint32_t *d_modnum = nullptr;
    uint8_t *d_seqs = nullptr;
    uint32_t *d_bA = nullptr;
    uint32_t *d_qA = nullptr;    // padded bucket starts (max_mass*scale + 1)
    uint32_t *d_qp = nullptr;    // query postings, qA[nb] words (+ kIaPad)
    uint16_t *d_qion = nullptr;  // ion of each query posting (same positions as d_qp)
    uint32_t *d_qAs = nullptr;   // search postings: bucket starts (multiples of 4)
    uint32_t *d_qps = nullptr;   // search postings (query postings less the classed y1 ones)
    uint8_t *d_cls = nullptr;    // per entry: its class
    uint64_t nsearch = 0;        // search postings (without padding)
    uint32_t *d_rows = nullptr;  // row table over the search postings (max_mass*scale buckets x stride)
    uint32_t stride = 0;
    bool built = false;
};

// Device scratch for one query call; grown on demand.
struct QueryScratch
{
    int2 *d_win = nullptr;        // nspec * nlen windows [minl, maxl]
    uint32_t *d_wide = nullptr;   // spectra that overflowed the packed scorecard
    uint32_t *d_nwide = nullptr;
    uint32_t *d_work = nullptr;   // work counters | cost-class counts | cursors
    uint32_t *d_order = nullptr;  // longest-first order | cost classes
    int32_t *d_fitstart = nullptr;  // first regression bin of each spectrum's tail fit (-1: none)
    size_t fit_cap = 0;
    size_t win_cap = 0, wide_cap = 0, order_cap = 0;
    // host-path staging
    void *d_in = nullptr;
    size_t in_cap = 0;
    void *d_outbuf = nullptr;
    size_t out_cap = 0;
};

// Caller-supplied scratch of one query (see launch_query_scratch).
struct ScratchPtrs
{
    int2 *win;          // nspec * nlen
    uint32_t *wide;     // nspec + 4
    uint32_t *work;     // 4 + 2 * 64
    uint32_t *order;    // 2 * nspec
    int32_t *fitstart;  // nspec
    LenDev *lens;       // HC_MAX_LENGTHS
};

// Per-query counters (device words): the searches' work counters, the
// overflow list's length, the small-window split point of the longest-first
// order, then its per-class counts and cursors.
constexpr uint32_t kWkSearch = 0, kWkWide = 1, kWkNwide = 2, kWkSmall = 3, kWkSplit = 4;
constexpr uint32_t kWkCnt = 8, kWkCur = kWkCnt + 64, kWorkWords = kWkCur + 64;

// What a captured query graph was recorded with; a call that differs re-captures.
struct GraphKey
{
    const void *idx, *moz, *inten, *prec, *dM, *out, *hist;
    const void *mlp, *learned;  // the learned form: network, learned log10 e-values (else null)
    float gate_resid;           // ... and its gate (kernel parameters of the captured graph)
    uint32_t gate_radius;
    uint32_t nspec, npeaks;
    hc_tuning tuning;
    uint32_t profiling;  // stage events captured or not
};

struct StreamStage;  // staging slots of hc_dslim_query_stream (hc_stream.cpp)
void free_stream_stage(StreamStage *s);

struct Launch
{
    uint32_t threads, tile, ctas_per_sm, pairs_per_warp;
    size_t smem;
    int grid;
};

}  // namespace hc

struct hc_ctx
{
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;     // per CTA, opt-in maximum
    size_t smem_sm = 0;        // per SM
    size_t smem_reserved = 0;  // per CTA, kept by the system
    hc_params p{};
    cudaStream_t stream = nullptr;
    hc_tuning tuning{};
    std::vector<hc::LenHost> lens;
    hc::LenDev *d_lens = nullptr;
    hc::IonTables tables{};
    hc::IonTables *d_tables = nullptr;
    // entry classes (shared by all lengths; ids are only ever added)
    std::vector<uint8_t> class_of;     // code -> class id
    hc::ClassKeys classes{};
    hc::ClassKeys *d_classes = nullptr;
    uint8_t *d_class_of = nullptr;
    hc::QueryConst *d_qconst = nullptr;
    hc::QueryScratch qs;
    std::string last_error;
    int last_launches = 0;
    bool lens_dirty = true;
    bool profiling = false;
    bool last_learned = false;  // the last query ran the learned tail (stage 5 recorded)
    cudaEvent_t ev[6] = {};  // windows | search | wide | tailfit | learned tail boundaries
    unsigned long long *d_phase = nullptr;  // per-phase SM cycles of the search kernel (diagnostics)
    double *d_log10 = nullptr;              // log10 table of the exact hyperscore path
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    hc::GraphKey graph_key{};
    int graph_launches = 0;
    hc::StreamStage *stage = nullptr;  // kept between streaming calls, grown on demand
};

namespace hc {

// What the device entry enumeration needs (passed by value to its kernels):
// the float residue and static-mod masses of UTILS_CalculatePepMass
// (utils.cpp:290-303), the residue -> mod-condition map and per-condition
// limits of MODS_ModList (mods.cpp:333-384), and each mod's mass as
// UTILS_CalculateModMass adds it (float(scaled mass) / float(scale)).
// Site bit of an N-terminal mod (an extension without a reference
// counterpart: a mod whose residue code is '^'); residues use bits 0..L-1.
constexpr int kNtermBit = 63;

struct EnumConst
{
    float aa[26];
    float stat[26];
    float h2o;
    int8_t cond_of[26];  // mod condition of a residue, -1 if none
    int8_t nterm;        // mod condition of the N-terminus ('^'), -1 if none
    uint32_t limit[HC_MAX_MODS];
    float modadd[HC_MAX_MODS];
    uint32_t vmods, nmods;
};

// hc_host.cpp
void make_enum_const(const hc_params &p, EnumConst *e);
void make_ion_tables(const hc_params &p, IonTables *t);
void make_query_const(QueryConst *q);
void make_log10_table(double *t, uint32_t n);
int64_t make_entries(const hc_params &p, uint32_t L, const uint8_t *seqs, uint32_t npep,
                     hc_entry *out, int64_t cap);
void division_magic(uint32_t d, uint32_t *magic, uint32_t *sh);

// hc_index.cu
int build_length_device(hc_ctx *ctx, LenHost &lh, const hc_entry *h_entries, bool sort_by_mass);
int build_query_postings(hc_ctx *ctx, LenHost &lh, const uint32_t *d_ids);
int build_rows(hc_ctx *ctx, LenHost &lh);  // entry classes, search postings and their row table
void class_keys_of(const hc_params &p, const IonTables &t, uint32_t code, uint32_t *keys);
int check_query_postings(hc_ctx *ctx, const LenHost &lh, uint64_t qtotal);
void free_len(LenHost &lh);
int export_ids(hc_ctx *ctx, const LenHost &lh, uint32_t *d_ids);

// hc_query.cu
uint32_t max_tile(const hc_ctx *ctx, uint32_t dF, uint32_t threads);
uint32_t max_tile_for(const hc_ctx *ctx, uint32_t dF, uint32_t ctas_per_sm, uint32_t threads);
int prepare_query(hc_ctx *ctx, uint32_t nspec);
size_t search_smem(uint32_t tile, uint32_t dF, bool wide, uint32_t threads);
// tailfit = false leaves the e-values to the learned tail (learned_pipeline)
int query_device(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_int,
                 const float *d_prec, const double *d_dM, uint32_t nspec, uint32_t npeaks,
                 hc_result *d_out, uint32_t *d_hist, cudaStream_t stream, bool tailfit = true);
// profiling: stage event i on st (a graph node when st is capturing)
cudaError_t record_stage(hc_ctx *ctx, int i, cudaStream_t st);
int tailfit_list(hc_ctx *ctx, hc_result *d_out, const uint32_t *d_hist, const uint32_t *list,
                 const uint32_t *d_nlist, uint32_t nmax, cudaStream_t st);
int sync_lengths(hc_ctx *ctx);
int preload_query_kernels(hc_ctx *ctx);
int launch_query_scratch(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_int,
                         const float *d_prec, const double *d_dM, uint32_t nspec, hc_result *d_out,
                         uint32_t *d_hist, const ScratchPtrs &s, cudaStream_t st);

// hc_mlp.cu: the learned tail after a search without tail fit
int learned_prepare(hc_mlp *m, uint32_t n);
void learned_gate(const hc_mlp *m, float *max_resid, uint32_t *radius);
int learned_pipeline(hc_mlp *m, const uint32_t *d_hist, hc_result *d_res, uint32_t n, float *lg, cudaStream_t st,
                     int *launches);

int set_error(hc_ctx *ctx, int code, const std::string &msg);
int cuda_check(hc_ctx *ctx, cudaError_t e, const char *what);

}  // namespace hc

#define HC_CUDA(ctx, call)                                          \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return hc::cuda_check((ctx), _e, #call); \
    } while (0)
