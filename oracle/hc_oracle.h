/*
 * CPU restatement of the HiCOPS DSLIM search path (TEST INFRASTRUCTURE).
 *
 * This is the oracle the GPU product is compared with, and the CPU baseline
 * that bench.py times. It is never linked into, loaded by, or
 * called from the product library. Every function restates one reference
 * function with the same arithmetic (types, evaluation order, truncations),
 * cited file:line inside the reference project (source/core/...).
 *
 * Parity of this restatement is pinned against the reference itself, compiled
 * from its own sources by oracle/ref/Makefile and run through
 * oracle/ref/ref_driver.cpp (tests/test_oracle_vs_reference.py, and the golden
 * vectors in tests/golden/ made by tests/golden/make_golden.py).
 *
 * One extension has no reference counterpart and so no pinned parity: a mod
 * whose residue code is "^" modifies the peptide's N-terminus (site bit 63,
 * the first mod of every b ion); the oracle restates the rules the product
 * defines for it, and is otherwise the reference's arithmetic unchanged.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_HIST_BINS 1002 /* 2 + MAX_HYPERSCORE*10 (source/core/dslim.cpp:419) */
#define ORC_MAX_MODS 15    /* MAX_MOD_TYPES (slm_dsts.h:28) */
#define ORC_MAXSHP 81      /* MAX_SHDPEAKS + 1 (utils.h:110) */
#define ORC_QALEN 100

/* flags: inputs on which the reference reads or writes out of bounds */
#define ORC_FLAG_LGFACT_OOB 0x1u  /* bc or yc > 80: lgfact[] read past its end (dslim_query.cpp:695) */
#define ORC_FLAG_HIST_OOB 0x2u    /* hyperscore bin > 1001 (dslim_query.cpp:719) */
#define ORC_FLAG_TAILFIT_OOB 0x4u /* tail-fit slice starts at index -1 (expeRT.cpp:653,690) */
#define ORC_FLAG_TAILFIT_EMPTY 0x8u /* empty tail-fit slice, 0/0 fit (expeRT.cpp:590-601) */

typedef struct orc_params
{
    uint32_t min_len, max_len, maxz, topmatches, scale, min_shp, min_cpsm;
    uint32_t min_mass, max_mass, dF;
    int32_t base_int, min_int;
    double dM, expect_max;
    uint32_t nmods, vmods_per_pep;
    uint32_t mod_mass[ORC_MAX_MODS];    /* scaled (uint) as hicops.cpp:661 */
    char mod_res[ORC_MAX_MODS][4];
    uint32_t mod_per_pep[ORC_MAX_MODS];
    uint32_t threads;
} orc_params;

/* One database entry (pepEntry, slm_dsts.h:146-282). */
typedef struct orc_entry
{
    float mass;
    uint32_t seqid;
    uint64_t sites;
    uint32_t modnum;
    uint32_t pad;
} orc_entry;

/* One peptide length's index (Index + SLMchunk, slm_dsts.h:306-356, nChunks = 1). */
typedef struct orc_length
{
    uint32_t L;
    uint32_t npep;
    uint32_t n;          /* entries */
    const uint8_t *seqs; /* npep * L residues */
    const orc_entry *entries;
    const uint32_t *bA;  /* max_mass*scale + 1 */
    const uint32_t *iA;  /* n * speclen */
} orc_length;

typedef struct orc_result
{
    uint32_t cpsms;
    int32_t idxoffset;
    int32_t psid;
    uint16_t sharedions;
    uint16_t totalions;
    float hyperscore;
    int32_t mu, beta;
    int32_t minhyp, nexthyp, maxhyp;
    uint32_t flags;
    uint32_t reported;
    double evalue;
    uint64_t post_bytes;
} orc_result;

float orc_pep_mass(const uint8_t *seq, uint32_t L);
float orc_mod_mass(const uint8_t *seq, uint32_t L, uint32_t modnum, const orc_params *p);
int orc_gen_spectrum(const uint8_t *seq, uint32_t L, const orc_entry *e, const orc_params *p,
                     uint32_t *keys);

/* Base entries then variants, in generation order; returns the count, or -1
 * if cap is too small. seqs: npep * L residues in file order. */
int64_t orc_make_entries(const uint8_t *seqs, uint32_t npep, uint32_t L, const orc_params *p,
                         orc_entry *out, int64_t cap);
void orc_sort_entries(orc_entry *e, uint32_t n); /* stable by mass */

int orc_build_index(const uint8_t *seqs, uint32_t L, const orc_entry *entries, uint32_t n,
                    const orc_params *p, uint32_t *bA, uint32_t *iA);

/* Query all spectra. dM_per_spec may be NULL. tie_rule 0 = the reference's
 * min-heap top (minheap.h:258-278); 1 = max hyperscore, then lowest
 * (length index, psid). hist: nspec*1002 u32 or NULL. */
int orc_query(const orc_length *lens, uint32_t nlen, const orc_params *p,
              const uint32_t *idx, const uint32_t *moz, const uint32_t *inten,
              const float *prec, const double *dM_per_spec, uint32_t nspec,
              int tie_rule, orc_result *out, uint32_t *hist, int threads);

/* Tail fit of one histogram (expeRT::ModelTailFit(Results*), expeRT.cpp:572-718). */
void orc_tailfit(const double *hist, int cpsms, int maxhyp, int32_t *mu, int32_t *beta,
                 int32_t *stt1, int32_t *end1, uint32_t *flags);

#ifdef __cplusplus
}
#endif
