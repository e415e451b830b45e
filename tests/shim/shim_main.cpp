// Test driver for hicops_gb300/shim/hicops_dslim_shim.cpp: it is compiled
// against the reference's headers and linked with libhicops_gb300.so, which
// checks the shim's types and layout assertions against the real Index,
// Queries, pepEntry and hCell. It supplies what the reference application
// would: the global gParams and DFile_PrintScore (recording its calls).
// Without a usable GPU the library reports HC_ERR_NO_DEVICE through the
// reference's status_t.
#include <cstdio>
#include <cstring>
#include <vector>

#include "dslim.h"
#include "dslim_fileout.h"

gParams params;
static int g_prints = 0;

status_t DFile_PrintScore(Index *, uint_t, float_t, hCell *, double_t, uint_t)
{
    g_prints++;
    return SLM_SUCCESS;
}

status_t DSLIM_Deinitialize();

int main()
{
    params.min_len = 7;
    params.max_len = 9;
    params.maxz = 2;
    params.dF = 2;
    params.dM = 100.0;
    params.threads = 1;
    params.vModInfo.num_vars = 1;
    params.vModInfo.vmods_per_pep = 2;
    params.vModInfo.vmods[0].residues[0] = 'M';
    params.vModInfo.vmods[0].modMass = 1599;
    params.vModInfo.vmods[0].aa_per_peptide = 2;
    // one length (8) with two peptides and their entries in mass order
    static char seqs[] = "PEPTIDEKMAGICMSK";
    Index idx;
    idx.pepIndex.seqs = seqs;
    idx.pepIndex.peplen = 8;
    idx.pepIndex.AAs = 16;
    idx.lclpepCnt = idx.pepCount = 2;
    std::vector<pepEntry> e(2);
    e[0].Mass = 927.45f;
    e[0].seqID = 0;
    e[1].Mass = 870.39f;
    e[1].seqID = 1;
    idx.pepEntries = e.data();
    idx.lcltotCnt = idx.totalCount = 2;
    const status_t c = DSLIM_Construct(&idx);
    Queries q;
    q.reset();
    q.rtimes = NULL;  // the constructor leaves it unset and the destructor deletes it (slm_dsts.h:444-456, 542)
    const status_t s = DSLIM_QuerySpectrum(&q, &idx, 1);
    const status_t d = DSLIM_Deinitialize();
    std::printf("construct %d query %d deinit %d prints %d\n", (int)c, (int)s, (int)d, g_prints);
    return 0;
}
