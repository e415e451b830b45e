/*
 * hicops_gb300 — GB300 (sm_103a) DSLIM database peptide search: C ABI.
 *
 * Drop-in boundary for the HiCOPS DSLIM index/query path. The reference calls
 * these C++ functions from its driver (source/app/hicops.cpp:287-340):
 *
 *   status_t DSLIM_Construct(Index *index);                     dslim.h:49
 *   status_t DSLIM_InitializeScorecard(Index *index, uint_t n); dslim.h:53
 *   status_t DSLIM_QuerySpectrum(Queries *ss, Index *index,
 *                                uint_t idxchunk);              dslim.h:184
 *   status_t DFile_PrintScore(Index*, uint_t specid, float_t pmass, hCell *psm,
 *                             double_t e_x, uint_t npsms);      dslim_fileout.h:29
 *
 * and read the global gParams (slm_dsts.h:359-418). Here every call takes a
 * context that owns the device-resident index, the parameters and the
 * scratch, and returns the reference's status_t convention (slmerr.h:24-46:
 * 0 = success, negative codes from -3001). Plain pointers and sizes only.
 *
 * Threading: one context per host thread; calls on one context are serialised
 * by the caller. Device work runs on the stream given (or the context's own).
 */
#ifndef HICOPS_GB300_H
#define HICOPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (slmerr.h:24-46) ---- */
#define HC_SUCCESS 0
#define HC_ERR_INVLD_MEMORY (-3001)
#define HC_ERR_INVLD_PARAM (-3002)
#define HC_ERR_INVLD_INDEX (-3003)
#define HC_ERR_INVLD_SIZE (-3004)
#define HC_ERR_FILE_NOT_FOUND (-3006)
#define HC_ERR_BAD_MEM_ALLOC (-3007)
#define HC_ERR_INVLD_PTR (-3008)
#define HC_ERR_INVLD_MOD (-3010)
#define HC_ERR_NOT_ENOUGH_DATA (-3012)
#define HC_ERR_FILE_ERROR (-3013)
/* codes without a reference counterpart */
#define HC_ERR_CUDA (-3020)      /* a CUDA runtime call failed; see hc_last_error */
#define HC_ERR_TIMEOUT (-3021)   /* hc_ctx_wait: the work was still running at the deadline */
#define HC_ERR_NO_DEVICE (-3022) /* no CUDA device, or not an sm_103 part */

#define HC_HIST_BINS 1002 /* 2 + MAX_HYPERSCORE*10 (dslim.cpp:419) */
#define HC_QALEN 100      /* peaks per spectrum (config.hpp QALEN) */
#define HC_MAX_MODS 15    /* MAX_MOD_TYPES (slm_dsts.h:28) */
#define HC_MAX_LENGTHS 64

/* per-spectrum result flags */
#define HC_FLAG_LGFACT_OOB 0x1u    /* bc or yc > 80: the reference reads lgfact[] out of bounds */
#define HC_FLAG_HIST_OOB 0x2u      /* hyperscore bin > 1001: out-of-bounds histogram write */
#define HC_FLAG_TAILFIT_OOB 0x4u   /* tail-fit slice starts at -1 (expeRT.cpp:653,690) */
#define HC_FLAG_TAILFIT_EMPTY 0x8u /* empty tail-fit slice: 0/0 fit (expeRT.cpp:590-601) */
#define HC_FLAG_WIDE 0x100u        /* scored by the wide-scorecard kernel */
#define HC_FLAG_LEARNED 0x200u     /* e-value from the learned tail (hc_dslim_query_learned) */

/* gParams fields on the DSLIM path (slm_dsts.h:359-418). dF is in bins
 * ((uint)(tolerance_Da * scale), hicops.cpp:564); dM in Da; mod_mass is scaled
 * ((uint)(mass * scale), hicops.cpp:661). mod_res holds the residue letters a
 * mod applies to; the code "^" (no reference counterpart) makes it a mod of
 * the peptide's N-terminus, recorded as site bit 63 of hc_entry.sites. */
typedef struct hc_params
{
    uint32_t min_len, max_len, maxz, topmatches, scale, min_shp, min_cpsm;
    uint32_t min_mass, max_mass, dF;
    int32_t base_int, min_int;
    double dM, expect_max;
    uint32_t nmods, vmods_per_pep;
    uint32_t mod_mass[HC_MAX_MODS];
    char mod_res[HC_MAX_MODS][4];
    uint32_t mod_per_pep[HC_MAX_MODS];
    uint32_t threads; /* host threads for host-side steps */
} hc_params;

/* One database entry: pepEntry (slm_dsts.h:146-282) with explicit padding. */
typedef struct hc_entry
{
    float mass;
    uint32_t seqid;
    uint64_t sites;
    uint32_t modnum;
    uint32_t pad;
} hc_entry;

/* Per-spectrum search result: the fields DFile_PrintScore receives
 * (dslim_fileout.cpp:112-152) plus the Results state (slm_dsts.h:694-754). */
typedef struct hc_result
{
    uint32_t cpsms;       /* candidate PSMs with hyperscore > 0 */
    int32_t idxoffset;    /* length index of the top hit (-1: none) */
    int32_t psid;         /* entry index of the top hit inside that length */
    uint16_t sharedions;  /* bc + yc of the top hit */
    uint16_t totalions;   /* speclen of the top hit */
    float hyperscore;     /* top hyperscore */
    int32_t mu, beta;     /* tail-fit slope/intercept x 1e6 (expeRT.cpp:703-704) */
    int32_t minhyp, nexthyp, maxhyp;
    uint32_t flags;
    uint32_t reported;    /* cpsms >= min_cpsm and evalue < expect_max */
    double evalue;
    uint64_t post_bytes;  /* algorithmic bytes: in-window postings + bucket reads */
} hc_result;

typedef struct hc_ctx hc_ctx;

/* Query-kernel launch shape (chosen by hc_tune or set by the caller). */
typedef struct hc_tuning
{
    uint32_t threads;      /* threads per CTA (multiple of 32, <= 1024) */
    uint32_t tile;         /* scorecard candidates per shared-memory tile */
    uint32_t ctas_per_sm;  /* resident CTAs per SM the grid is sized for */
    uint32_t pairs_per_warp; /* 16-byte postings chunks (4 postings each) a lane keeps
                                in flight: 1, 2, 4 or 8 */
    uint32_t schedule;     /* 0: persistent CTAs, work stealing in batch order;
                              1: plain, one CTA per spectrum;
                              2: batched, persistent CTAs, longest windows first */
    uint32_t defer_cap;    /* candidates per spectrum whose hyperscore sign or histogram
                              bin the float estimate leaves open, queued for one exact
                              evaluation at the spectrum's end (<= HC_DEFER_MAX; 0: each
                              is evaluated in place). Results do not depend on it. */
    uint32_t small_log2;   /* schedule 2: spectra whose windows hold fewer than
                              2^small_log2 candidates in all run in a second launch of
                              128-thread CTAs, several per SM, after the others (0: none;
                              at most 40). Results do not depend on it. */
} hc_tuning;
#define HC_DEFER_MAX 128

int hc_version(void);
const char *hc_status_string(int status);

/* ---- context (owns the index, the scorecard scratch and a stream) ---- */
int hc_ctx_create(int device, const hc_params *p, hc_ctx **out);
int hc_ctx_destroy(hc_ctx *ctx);
const char *hc_last_error(const hc_ctx *ctx);
int hc_ctx_set_tuning(hc_ctx *ctx, const hc_tuning *t);
int hc_ctx_get_tuning(const hc_ctx *ctx, hc_tuning *t);
/* Waits at most timeout_s seconds (< 0: no limit) for the device work
 * enqueued on `stream` (cudaStream_t; NULL = the context stream), e.g. by
 * hc_dslim_query_device. HC_SUCCESS: it has finished; HC_ERR_TIMEOUT: it was
 * still running at the deadline (nothing is cancelled: wait again later);
 * HC_ERR_CUDA: it failed. Replaces the reference's unbounded wait for a
 * batch (the manager thread joining DSLIM_QuerySpectrum, dslim_query.cpp:361)
 * for callers that serve requests with deadlines. */
int hc_ctx_wait(hc_ctx *ctx, void *stream, double timeout_s);

/* ---- index (DSLIM_Construct, dslim.h:49; LBE_Initialize, lbe.h) ----
 * Builds the SLM index of one peptide length on the device: entries (base
 * peptides in file order, then variable-mod variants, mods.cpp:333-496) are
 * enumerated and sorted by mass on the device (stable), ion keys are generated, and the
 * bucket (bA) and postings (iA) arrays are built by a device radix sort.
 * seqs: npep*L residues (already mass-filtered as LBE_CountPeps does,
 * lbe_internal.cpp:413). order: optional entries in a caller-fixed order
 * (e.g. the reference's own sorted order); NULL = device sort. */
int hc_dslim_construct(hc_ctx *ctx, uint32_t L, const uint8_t *seqs, uint32_t npep,
                       const hc_entry *order, uint32_t norder);
/* Loads a host-built index as-is (bA/iA as DSLIM_Construct lays them out). */
int hc_dslim_load(hc_ctx *ctx, uint32_t L, const uint8_t *seqs, uint32_t npep,
                  const hc_entry *entries, uint32_t n, const uint32_t *bA, const uint32_t *iA);
int hc_dslim_info(hc_ctx *ctx, uint32_t L, uint32_t *n_entries, uint64_t *n_postings);
/* Copies one length's entries / bA (max_mass*scale+1) / iA back (any may be NULL). */
int hc_dslim_export(hc_ctx *ctx, uint32_t L, hc_entry *entries, uint32_t *bA, uint32_t *iA);
/* Enumerates a length's entries on the host exactly as hc_dslim_construct
 * does before its device sort; returns the count (or a negative status).
 * out may be NULL to count only. */
int64_t hc_make_entries(const hc_params *p, uint32_t L, const uint8_t *seqs, uint32_t npep,
                        hc_entry *out, int64_t cap);

/* ---- query (DSLIM_QuerySpectrum, dslim.h:184) ----
 * CSR batch in host memory: idx[nspec+1] offsets into moz/intensity;
 * precurse[nspec]; dM_per_spec optional per-spectrum tolerance (Da, NULL =
 * params.dM). out[nspec] results; hist optional nspec*1002 counts. */
int hc_dslim_query(hc_ctx *ctx, const uint32_t *idx, const uint32_t *moz,
                   const uint32_t *intensity, const float *precurse,
                   const double *dM_per_spec, uint32_t nspec, hc_result *out, uint32_t *hist);
/* Same, all buffers device-resident, enqueued on `stream` (cudaStream_t;
 * NULL = the context stream). npeaks = idx[nspec]. Returns after enqueueing;
 * the host does not wait. */
int hc_dslim_query_device(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz,
                          const uint32_t *d_intensity, const float *d_precurse,
                          const double *d_dM, uint32_t nspec, uint32_t npeaks,
                          hc_result *d_out, uint32_t *d_hist, void *stream);
/* Batched form: the same pipeline captured once into a CUDA graph and
 * replayed; a call whose buffers, sizes or tuning differ from the captured
 * one re-captures. Results are identical to hc_dslim_query_device. */
int hc_dslim_query_graph(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz,
                         const uint32_t *d_intensity, const float *d_precurse,
                         const double *d_dM, uint32_t nspec, uint32_t npeaks,
                         hc_result *d_out, uint32_t *d_hist, void *stream);
/* Allocation-free form of hc_dslim_query_device (no reference counterpart):
 * same arguments and results, but its scratch is a fixed file-scope device
 * array, so it never allocates, for callers that may not allocate device
 * memory while they search. At most 16384 spectra per call (larger batches
 * return HC_ERR_INVLD_SIZE). The first call in a CUDA context (normally the
 * device's primary context) does the set-up: it looks up the scratch address
 * and loads every kernel the search can launch, so that later calls load no
 * code; make it before any stream capture. All calls on one device share the
 * scratch: calls that overlap on the GPU race. */
int hc_dslim_query_noalloc(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz,
                           const uint32_t *d_intensity, const float *d_precurse,
                           const double *d_dM, uint32_t nspec, uint32_t npeaks,
                           hc_result *d_out, uint32_t *d_hist, void *stream);
/* Autotuner: times the search on a device-resident sample batch for every
 * launch shape of a small grid (schedule x CTAs per SM x block size x chunks
 * in flight per lane, each with the largest scorecard tile that fits), then
 * smaller tiles (1, 2 and 4 row-table blocks fewer) for the three fastest,
 * keeps the fastest in the context and returns it. */
int hc_tune(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_intensity,
            const float *d_precurse, const double *d_dM, uint32_t nspec, uint32_t npeaks,
            hc_result *d_out, uint32_t *d_hist, hc_tuning *best, float *best_ms);
/* ---- learned e-value tail (no reference counterpart; replaces the
 * per-spectrum regression of expeRT::ModelTailFit, expeRT.cpp:572-718, which
 * stays the fallback and the yardstick) ----
 * A 256 -> 128 -> 64 -> 4 FP32 MLP mapping a spectrum's histogram (as its log
 * survival curve, bins >= 255 folded) to the tail line (slope, intercept),
 * the first bin of the regression window and the line's RMS residual.
 * Parameters: W1[256x128] b1 W2[128x64] b2 W3[64x4] b3. A spectrum whose
 * predicted residual is within the gate gets its e-value from the network's
 * window: the predicted first bin is confirmed on the FP32 survival curve
 * (the bin before the first point at or below expeRT's 22 % level, tested
 * for the prediction and its neighbours within the radius), the window ends
 * at expeRT's 87 % cut (expeRT.cpp:646-676), the line is the FP32
 * least-squares fit over it and e = 10^(line at the top hit) * cpsms. Every
 * other spectrum gets the expeRT fit. */
typedef struct hc_mlp hc_mlp;
int hc_mlp_create(hc_ctx *ctx, uint64_t seed, hc_mlp **out);
int hc_mlp_destroy(hc_mlp *m);
int hc_mlp_num_params(void);
int hc_mlp_get_params(hc_mlp *m, float *host);
int hc_mlp_set_params(hc_mlp *m, const float *host);
/* Gate: the largest predicted RMS residual (log10 units; 0.1 by default) of
 * a learned spectrum, and the radius (0..15, 4 by default) of first bins
 * tested on either side of the predicted one. */
int hc_mlp_set_gate(hc_mlp *m, float max_resid, uint32_t radius);
int hc_mlp_get_gate(const hc_mlp *m, float *max_resid, uint32_t *radius);
/* X[n,256] from the histograms and results of a query (device buffers). */
int hc_mlp_features(hc_ctx *ctx, const uint32_t *d_hist, const hc_result *d_res, uint32_t n, float *d_X,
                    void *stream);
/* Y[n,4] = the training targets from expeRT's own window (found by a full
 * search of the curve): slope, intercept, first bin, RMS residual of the line
 * over the window; NaN (no target, no loss) where there is no such fit. */
int hc_mlp_targets(hc_ctx *ctx, const uint32_t *d_hist, const hc_result *d_res, uint32_t n, float *d_Y,
                   void *stream);
/* out[n,4] = the network's outputs (scaled: slope x 10, intercept / 4, first
 * bin / 10, residual x 5). */
int hc_mlp_forward(hc_mlp *m, const float *d_X, uint32_t n, float *d_out, void *stream);
/* Gradients of the mean squared error (scaled targets) over one batch, to host. */
int hc_mlp_gradients(hc_mlp *m, const float *d_X, const float *d_Y, uint32_t n, float *host_grads,
                     float *loss);
/* Adam training over [0, n) in minibatches of `batch` for `epochs`. */
int hc_mlp_train(hc_mlp *m, const float *d_X, const float *d_Y, uint32_t n, uint32_t batch,
                 uint32_t epochs, float lr, float *final_loss);
/* Every spectrum's learned log10 e-value with no residual gate and no result
 * written (NaN where no first bin was confirmed): d_aux[3n] = {predicted
 * residual, residual of the line, offset of the confirmed first bin from the
 * prediction}. baseline != 0 uses no network: the search starts at the
 * curve's first point (d_X unused). */
int hc_mlp_tail_probe(hc_mlp *m, const float *d_X, const uint32_t *d_hist, const hc_result *d_res, uint32_t n,
                      int baseline, float *d_learned_log10e, float *d_aux, void *stream);
/* Batched+learned query: the search (as hc_dslim_query_graph) without the
 * tail fit, then features, network, learned e-values where the gates pass,
 * and the expeRT fit (k_tailfit) only on the spectra left over, all captured
 * once into a CUDA graph and replayed (a call whose buffers, sizes, tuning or
 * network differ re-captures). Learned spectra carry HC_FLAG_LEARNED and
 * their line in mu / beta; integer fields equal hc_dslim_query_device's.
 * d_learned_log10e (optional, nspec floats): learned log10 e-values (NaN where
 * expeRT's fit was used). */
int hc_dslim_query_learned(hc_ctx *ctx, hc_mlp *mlp, const uint32_t *d_idx, const uint32_t *d_moz,
                           const uint32_t *d_intensity, const float *d_precurse, const double *d_dM,
                           uint32_t nspec, uint32_t npeaks, hc_result *d_out, uint32_t *d_hist,
                           float *d_learned_log10e, void *stream);
/* ---- on-disk index (no reference counterpart: the reference rebuilds its
 * index on every run, hicops.cpp:174-260) ----
 * hc_dslim_save writes every built length (entries, sequences, bucket offsets
 * and the device postings with their ions) to one file with a hash of the index-defining
 * parameters; hc_dslim_restore reads it into a context created with the same
 * parameters (else HC_ERR_INVLD_PARAM) and rebuilds the derived row tables.
 * HC_ERR_FILE_NOT_FOUND / HC_ERR_FILE_ERROR on I/O failures. */
int hc_dslim_save(hc_ctx *ctx, const char *path);
int hc_dslim_restore(hc_ctx *ctx, const char *path);

/* ---- PSM output (DFile_PrintScore, dslim_fileout.cpp:112-152; header 68-72) ----
 * Writes one TSV row per reported spectrum (reported != 0) with the
 * reference's columns: file, scan_num (spec_base + i + 1), prec_mass, charge,
 * retention_time, peptide, matched_ions, total_ions, calc_pep_mass, mass_diff,
 * mod_info (empty, as in the reference), hyperscore, expectscore, num_hits;
 * numbers as std::to_string prints them. The header is written unless
 * `append`. charges / rtimes may be NULL (printed as 0). */
int hc_write_psms(hc_ctx *ctx, const char *path, const char *file_label, uint32_t spec_base,
                  const hc_result *res, uint32_t nspec, const float *precurse, const int32_t *charges,
                  const float *rtimes, int append);

/* ---- MS2 ingestion (MSQuery, source/core/msquery.cpp) ----
 * hc_ms2_open replaces MSQuery::initialize (msquery.cpp:88-178) and reads the
 * whole file once as MSQuery::readspectrum reads it spectrum by spectrum
 * (msquery.cpp:300-505): one spectrum per 'S' line; 'Z' lines give the charge
 * and precursor, 'I RTime' lines the retention time, every other non-empty
 * line not starting with 'H' or 'D' a peak, m/z scaled by the context's
 * `scale` and intensity by 1000, truncated to integers. *nspec = number of
 * spectra, *maxslen = largest raw peak count. HC_ERR_FILE_ERROR when the file
 * cannot be opened or read, HC_ERR_INVLD_SIZE when it holds no peak at all
 * (the reference's ERR_INVLD_SIZE). */
typedef struct hc_ms2 hc_ms2;
int hc_ms2_open(hc_ctx *ctx, const char *path, hc_ms2 **out, uint32_t *nspec, uint32_t *maxslen);
/* The same without a context (host only, no CUDA call): m/z scaled by `scale`.
 * The file is read once and parsed by all host threads in stretches that
 * start at 'S' lines; a spectrum without its own 'Z' / 'I RTime' line
 * inherits the previous one's values, as MSQuery's single spectrum_t does.
 * Returns the status code only (no context to hold a message). */
int hc_ms2_read(const char *path, uint32_t scale, hc_ms2 **out, uint32_t *nspec, uint32_t *maxslen);
/* The raw spectra [first, first+count) as readspectrum leaves them (before
 * pickpeaks): off[count+1] (relative), mz / intensity (the raw peaks in file
 * order), prec, z (unsigned, as spectrum_t holds it), rtime; NULL skips an
 * array. */
int hc_ms2_raw(const hc_ms2 *m, uint32_t first, uint32_t count, uint64_t *off, uint32_t *mz, uint32_t *intensity,
               double *prec, uint32_t *z, double *rtime);
/* Replaces MSQuery::extractbatch (msquery.cpp:239-297) and pickpeaks
 * (msquery.cpp:509-569): spectra [first, first+count) clamped to the file's
 * end (*nout = how many) are peak-picked on the device (quicksort by
 * intensity with the reference's tie order, top peak = base_int, at most
 * HC_QALEN kept, those >= min_int) into the CSR batch idx[*nout+1],
 * moz / intensity (room for *nout * HC_QALEN each), precurse, charges
 * (MAX(1, Z)), rtimes (MAX(0, rtime)); *npeaks = idx[*nout]. The batch
 * layout is the reference's Queries (slm_dsts.h:422-559), ready for
 * hc_dslim_query. */
int hc_ms2_extract(hc_ctx *ctx, hc_ms2 *m, uint32_t first, uint32_t count, uint32_t *idx, uint32_t *moz,
                   uint32_t *intensity, float *precurse, int32_t *charges, float *rtimes, uint32_t *nout,
                   uint64_t *npeaks);
/* Replaces MSQuery::DeinitQueryFile (msquery.cpp:571-605). */
int hc_ms2_close(hc_ms2 *m);

/* ---- streaming query over a large host batch ----
 * Replaces the batch loop of DSLIM_SearchManager (dslim_query.cpp:160-420),
 * where an I/O thread fills QCHUNK-sized batches that DSLIM_QuerySpectrum
 * searches one after another. The host batch (any host memory, CSR as in
 * hc_dslim_query) is cut into sub-batches of `batch` spectra that alternate
 * between two pinned/device staging slots, so the copies of one sub-batch
 * overlap the search of the other. The slots belong to the context and are
 * kept between calls (grown when a call needs more room). With `mlp`
 * non-null every sub-batch gets the learned tail (as hc_dslim_query_learned)
 * and learned_log10e (optional, nspec floats) receives its values. hist
 * (optional) receives nspec*HC_HIST_BINS counts. Synchronous: returns when
 * every result is in `out`. */
int hc_dslim_query_stream(hc_ctx *ctx, const uint32_t *idx, const uint32_t *moz, const uint32_t *intensity,
                          const float *precurse, const double *dM, uint32_t nspec, uint32_t batch,
                          hc_mlp *mlp, hc_result *out, uint32_t *hist, float *learned_log10e);
/* Diagnostics: with phase timing on, the search kernel adds up SM clock
 * cycles per phase (bucket setup, postings stream, score pass 1, score pass 2,
 * tile clear, rest) over all CTAs, then four counts (tiles, tiles scored by a
 * whole-tile scan, listed candidates, exact hyperscores in pass 1);
 * hc_phase_cycles returns and clears them. */
int hc_ctx_set_phase_timing(hc_ctx *ctx, int on);
int hc_phase_cycles(hc_ctx *ctx, uint64_t out[10]);
/* Host-side check of the postings-id decoding: counts x in [0, xmax) for
 * which the multiply-shift quotient used on the device differs from x / d
 * (0 expected; no device needed). */
uint64_t hc_check_division(uint32_t d, uint32_t xmax);
/* Kernel launches made by the last query call (for launch accounting). */
int hc_last_launch_count(const hc_ctx *ctx);
/* With profiling on, every query records CUDA events around its kernels on
 * the query stream; hc_last_kernel_times waits for the last query and
 * returns the device time of each stage in ms (window search, packed search,
 * wide search, tail fit). */
int hc_ctx_set_profiling(hc_ctx *ctx, int on);
int hc_last_kernel_times(hc_ctx *ctx, float *ms_windows, float *ms_search, float *ms_wide,
                         float *ms_tailfit);
/* The same as ms[0..3], plus ms[4] = the learned tail (features, network,
 * learned e-values and the fallback tail fit) when the last query ran it;
 * *nstages = 5 then, else 4 (and the tail fit is ms[3]). */
int hc_last_stage_times(hc_ctx *ctx, float *ms, int *nstages);

#ifdef __cplusplus
}
#endif
#endif /* HICOPS_GB300_H */
