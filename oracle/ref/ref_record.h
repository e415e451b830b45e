/*
 * Record layout written by the reference-oracle driver (TEST INFRASTRUCTURE).
 * One record per query spectrum; `reported` is 0 when the reference did not
 * call DFile_PrintScore for it (cpsms < min_cpsm or e >= expect_max,
 * source/core/dslim_query.cpp:773,812).
 * The Python side reads it with the numpy dtype in tests/golden/make_golden.py.
 */
#pragma once
#include <stdint.h>

#define REF_HIST_BINS 1002 /* 2 + MAX_HYPERSCORE*10, source/core/dslim.cpp:419 */

typedef struct ref_record
{
    int32_t reported;
    int32_t psid;
    int32_t idxoffset;
    int32_t sharedions;
    int32_t totalions;
    float hyperscore;
    double e_x;
    int32_t npsms;
    int32_t mu;
    int32_t beta;
    int32_t minhyp;
    int32_t nexthyp;
    int32_t maxhyp;
    uint32_t seqid;
    uint32_t modnum;
    uint64_t sites;
    float pepmass;
    uint32_t pad;
    uint32_t hist[REF_HIST_BINS];
    uint32_t pad2[2];
} ref_record_t;
