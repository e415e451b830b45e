/*
 * CPU restatement of the HiCOPS DSLIM search path (TEST INFRASTRUCTURE).
 * See hc_oracle.h. Compiled with -ffp-contract=off so that every product and
 * sum rounds as on x86-64 (the reference's own build platform).
 */
#include "hc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* site bit of an N-terminal mod (extension; residues use bits 0..L-1) */
#define ORC_NTERM_BIT 63

/* ---------------------------------------------------------------------- */
/* constants: source/core/utils.cpp:28-101                                  */
/* ---------------------------------------------------------------------- */
#define ORC_H2O 18.015f
#define ORC_PROTON 1.00727647
#define ORC_NAA -20000

static const float AAMass[26] = {
    71.03712f, ORC_NAA, 103.00919f, 115.030f, 129.0426f, 147.068f, 57.02146f,
    137.060f, 113.084f, ORC_NAA, 128.094f, 113.084f, 131.0405f, 114.043f,
    ORC_NAA, 97.0527f, 128.05858f, 156.1012f, 87.032f, 101.0476f, ORC_NAA,
    99.06841f, 186.0793f, ORC_NAA, 163.0633f, ORC_NAA};
static const float StatMods[26] = {0, 0, 57.021464f, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                   0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};

/* GETAA(x, z), utils.cpp:101: float + float, then + PROTON*z in double */
static inline double getaa(uint8_t x, double z)
{
    float s = AAMass[x - 'A'] + StatMods[x - 'A'];
    return (double)s + ORC_PROTON * z;
}

/* x86-64 cvttsd2si: truncation, INT_MIN for NaN or out of range. The
 * reference converts the fit slope/intercept this way (expeRT.cpp:703-704). */
static inline int32_t x86_d2i(double v)
{
    if (!(v > -2147483649.0 && v < 2147483648.0))
        return (int32_t)0x80000000u;
    return (int32_t)v;
}

/* UTILS_CalculatePepMass, utils.cpp:290-303 */
float orc_pep_mass(const uint8_t *seq, uint32_t L)
{
    float mass = ORC_H2O;
    for (uint32_t l = 0; l < L; l++)
    {
        mass += AAMass[seq[l] - 'A'];
        mass += StatMods[seq[l] - 'A'];
    }
    return mass;
}

/* UTILS_CalculateModMass, utils.cpp:337-362. The loop there shifts by `start`
 * (0xF0 after the first round) instead of by 4; the shift count is taken mod
 * 32 by the hardware, (modNum & 0xF0) >> 16 is 0, so exactly the first mod's
 * mass is added. */
float orc_mod_mass(const uint8_t *seq, uint32_t L, uint32_t modnum, const orc_params *p)
{
    float mass = orc_pep_mass(seq, L);
    uint32_t first = modnum & 0x0F;
    if (first != 0)
        mass += ((float)p->mod_mass[first - 1] / (float)p->scale);
    return mass;
}

/* UTILS_GenerateSpectrum (utils.cpp:231-276) and UTILS_GenerateModSpectrum
 * (utils.cpp:378-505), followed by the legality rules of DSLIM_ConstructChunk
 * (dslim.cpp:296-323): ions >= max_mass*scale clamp to max_mass*scale-1,
 * entries outside [min_mass, max_mass] get all-zero keys. Returns 1 when the
 * mod spectrum would be read uninitialised (mass exactly on a bound). */
int orc_gen_spectrum(const uint8_t *seq, uint32_t L, const orc_entry *e, const orc_params *p,
                     uint32_t *S)
{
    const uint32_t maxz = p->maxz, scale = p->scale;
    const uint32_t speclen = 2 * maxz * (L - 1);
    const double minmass = p->min_mass, maxmass = p->max_mass;
    int uninit = 0;
    float mass;

    if (e->modnum == 0)
    {
        mass = orc_pep_mass(seq, L);
        if (mass > 0)
        {
            memset(S, 0, sizeof(uint32_t) * speclen);
            for (uint32_t z = 0; z < maxz; z++)
            {
                uint32_t bs = z * (L - 1), ys = z * (L - 1) + maxz * (L - 1);
                S[bs] = (uint32_t)((getaa(seq[0], z + 1) * scale) / (z + 1));
                S[ys] = (uint32_t)(((getaa(seq[L - 1], z + 1) + ORC_H2O) * scale) / (z + 1));
                for (uint32_t l = 1; l < L - 1; l++)
                {
                    S[bs + l] = S[bs + l - 1] + (uint32_t)((getaa(seq[l], 0) * scale) / (z + 1));
                    S[ys + l] = S[ys + l - 1] + (uint32_t)((getaa(seq[L - 1 - l], 0) * scale) / (z + 1));
                }
            }
        }
    }
    else
    {
        mass = orc_mod_mass(seq, L, e->modnum, p);
        if (mass > minmass && mass < maxmass)
        {
            int modNums[ORC_MAX_MODS];
            int modSeen = 0;
            uint32_t bm = e->modnum;
            for (int i = 0; i < ORC_MAX_MODS; i++)
            {
                modNums[i] = (int)(bm & 0x0F) - 1;
                bm /= 16;
                if (modNums[i] != -1)
                    modSeen++;
            }
            for (uint32_t z = 0; z < maxz; z++)
            {
                uint32_t bs = z * (L - 1), ys = z * (L - 1) + maxz * (L - 1);
                S[bs] = (uint32_t)(getaa(seq[0], z + 1) * scale);
                S[ys] = (uint32_t)((getaa(seq[L - 1], z + 1) + ORC_H2O) * scale);
                for (uint32_t l = 1; l < L - 1; l++)
                {
                    S[bs + l] = S[bs + l - 1] + (uint32_t)(getaa(seq[l], 0) * scale);
                    S[ys + l] = S[ys + l - 1] + (uint32_t)(getaa(seq[L - 1 - l], 0) * scale);
                }
            }
            for (uint32_t z = 0; z < maxz; z++)
            {
                /* an N-terminal mod (extension) is the first mod of every b ion */
                uint32_t bs = z * (L - 1), counter = (uint32_t)((e->sites >> ORC_NTERM_BIT) & 1ull);
                for (uint32_t l = 0; l < L - 1; l++)
                {
                    counter += (e->sites >> l) & 1ull;
                    for (uint32_t k = 0; k < counter; k++)
                        S[bs + l] += p->mod_mass[modNums[k]];
                    S[bs + l] /= (z + 1);
                }
            }
            for (uint32_t z = 0; z < maxz; z++)
            {
                uint32_t ys = z * (L - 1) + maxz * (L - 1), counter = 0;
                for (int l = (int)L - 1; l > 0; l--)
                {
                    counter += (e->sites >> l) & 1ull;
                    for (uint32_t k = 0; k < counter; k++)
                        S[ys + (L - 1) - l] += p->mod_mass[modNums[modSeen - 1 - (int)k]];
                    S[ys + (L - 1) - l] /= (z + 1);
                }
            }
        }
        else if (mass >= minmass && mass <= maxmass)
        {
            uninit = 1;
            memset(S, 0, sizeof(uint32_t) * speclen);
        }
    }

    if (mass >= minmass && mass <= maxmass)
    {
        const uint32_t top = (uint32_t)(maxmass * scale);
        for (uint32_t i = 0; i < speclen; i++)
            if (S[i] >= maxmass * scale)
                S[i] = top - 1;
    }
    else
        memset(S, 0, sizeof(uint32_t) * speclen);
    return uninit;
}

/* ---------------------------------------------------------------------- */
/* entries: LBE_GeneratePeps (lbe_internal.cpp:204-229) and MODS_ModList    */
/* (mods.cpp:333-384) in depth-first order                                  */
/*                                                                          */
/* Extension without a reference counterpart: a mod whose residue code is  */
/* '^' modifies the peptide's N-terminus. The walk then runs over virtual   */
/* positions v = 0..L, v = 0 the N-terminus (site bit 63) and v >= 1        */
/* residue v-1 (site bit v-1); without such a mod, v = 0 is never           */
/* modifiable and the walk is MODS_ModList's.                               */
/* ---------------------------------------------------------------------- */
typedef struct
{
    const orc_params *p;
    int cond_of[26];
    int nterm; /* mod index of the N-terminal mod, -1 if none */
    const uint8_t *seq;
    uint32_t L;
    uint32_t seqid;
    orc_entry *out;
    int64_t n, cap;
} modgen_t;

static void modlist(modgen_t *g, const int *conds, int total, uint64_t sites, uint32_t modnum,
                    int v, int novel, int modsSeen)
{
    if (novel)
    {
        if (g->n < g->cap)
        {
            orc_entry *e = &g->out[g->n];
            e->seqid = g->seqid;
            e->sites = sites;
            e->modnum = modnum;
            e->pad = 0;
            e->mass = orc_mod_mass(g->seq, g->L, modnum, g->p);
        }
        g->n++;
    }
    if (total == 0 || v > (int)g->L)
        return;
    const int c = v == 0 ? g->nterm : g->cond_of[g->seq[v - 1] - 'A'];
    const int bit = v == 0 ? ORC_NTERM_BIT : v - 1;
    if (c != -1 && conds[c] > 0)
    {
        int dup[ORC_MAX_MODS];
        memcpy(dup, conds, sizeof(dup));
        dup[c] -= 1;
        modlist(g, dup, total - 1, sites | (1ull << bit),
                modnum + (uint32_t)((1u << (4 * modsSeen)) * (uint32_t)(1 + c)), v + 1, 1,
                modsSeen + 1);
    }
    modlist(g, conds, total, sites, modnum, v + 1, 0, modsSeen);
}

int64_t orc_make_entries(const uint8_t *seqs, uint32_t npep, uint32_t L, const orc_params *p,
                         orc_entry *out, int64_t cap)
{
    modgen_t g;
    memset(&g, 0, sizeof(g));
    g.p = p;
    g.L = L;
    g.out = out;
    g.cap = cap;
    for (int i = 0; i < 26; i++)
        g.cond_of[i] = -1;
    g.nterm = -1;
    for (uint32_t m = 0; m < p->nmods; m++)
        for (int j = 0; j < 4 && p->mod_res[m][j]; j++)
        {
            const int c = p->mod_res[m][j] - 'A';
            if (p->mod_res[m][j] == '^')
                g.nterm = (int)m;
            else if (c >= 0 && c < 26)
                g.cond_of[c] = (int)m;
        }
    for (uint32_t i = 0; i < npep; i++)
    {
        if (g.n < cap)
        {
            out[g.n].mass = orc_pep_mass(seqs + (size_t)i * L, L);
            out[g.n].seqid = i;
            out[g.n].sites = 0;
            out[g.n].modnum = 0;
            out[g.n].pad = 0;
        }
        g.n++;
    }
    if (p->vmods_per_pep > 0 && p->nmods > 0)
    {
        int conds[ORC_MAX_MODS] = {0};
        for (uint32_t m = 0; m < p->nmods; m++)
            conds[m] = (int)p->mod_per_pep[m];
        for (uint32_t i = 0; i < npep; i++)
        {
            g.seq = seqs + (size_t)i * L;
            g.seqid = i;
            modlist(&g, conds, (int)p->vmods_per_pep, 0, 0, 0, 0, 0);
        }
    }
    return g.n <= cap ? g.n : -1;
}

static int cmp_entry_mass(const void *a, const void *b)
{
    const orc_entry *x = (const orc_entry *)a, *y = (const orc_entry *)b;
    if (x->mass < y->mass) return -1;
    if (x->mass > y->mass) return 1;
    return 0;
}

/* Stable merge sort by mass (the reference uses std::sort, lbe_internal.cpp:186,
 * whose order among equal masses is unspecified). */
void orc_sort_entries(orc_entry *e, uint32_t n)
{
    orc_entry *tmp = (orc_entry *)malloc(sizeof(orc_entry) * (n ? n : 1));
    for (uint32_t w = 1; w < n; w *= 2)
    {
        for (uint32_t lo = 0; lo < n; lo += 2 * w)
        {
            uint32_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
            uint32_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi)
                tmp[k++] = (cmp_entry_mass(&e[j], &e[i]) < 0) ? e[j++] : e[i++];
            while (i < mid) tmp[k++] = e[i++];
            while (j < hi) tmp[k++] = e[j++];
        }
        memcpy(e, tmp, sizeof(orc_entry) * n);
    }
    free(tmp);
}

/* ---------------------------------------------------------------------- */
/* index: DSLIM_ConstructChunk (dslim.cpp:216-347), the bA scan (97-125),   */
/* DSLIM_SLMTransform (361-388) and DSLIM_Optimize (452-482). The key/value */
/* quicksort followed by the per-bucket sort leaves, in every bucket, the   */
/* ion ids in ascending order: restated here as a stable counting sort.     */
/* ---------------------------------------------------------------------- */
int orc_build_index(const uint8_t *seqs, uint32_t L, const orc_entry *entries, uint32_t n,
                    const orc_params *p, uint32_t *bA, uint32_t *iA)
{
    const uint32_t speclen = 2 * p->maxz * (L - 1);
    const uint32_t nb = p->max_mass * p->scale;
    const size_t total = (size_t)n * speclen;
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * (total ? total : 1));
    int uninit = 0;
#pragma omp parallel for schedule(static) reduction(+ : uninit)
    for (int64_t k = 0; k < (int64_t)n; k++)
        uninit += orc_gen_spectrum(seqs + (size_t)entries[k].seqid * L, L, &entries[k], p,
                                   keys + (size_t)k * speclen);
    memset(bA, 0, sizeof(uint32_t) * (nb + 1));
    for (size_t i = 0; i < total; i++)
        bA[keys[i]]++;
    uint32_t run = 0;
    for (uint32_t b = 0; b <= nb; b++)
    {
        uint32_t c = bA[b];
        bA[b] = run;
        run += (b < nb) ? c : 0;
    }
    uint32_t *cur = (uint32_t *)malloc(sizeof(uint32_t) * (nb + 1));
    memcpy(cur, bA, sizeof(uint32_t) * (nb + 1));
    for (size_t i = 0; i < total; i++)
        iA[cur[keys[i]]++] = (uint32_t)i;
    free(cur);
    free(keys);
    return uninit;
}

/* ---------------------------------------------------------------------- */
/* minHeap<hCell> (minheap.h:86-278) keyed on the float hyperscore          */
/* ---------------------------------------------------------------------- */
typedef struct
{
    float h;
    int32_t ixx, psid;
    uint16_t shp, tot;
} hcell;

typedef struct
{
    int size, cap;
    hcell a[64];
} heap_t;

static void heapify(heap_t *H, int pos)
{
    for (;;)
    {
        int r = (pos + 1) * 2, l = r - 1, s = pos;
        float sv = H->a[s].h;
        if (l < H->size && H->a[l].h < sv) { s = l; sv = H->a[l].h; }
        if (r < H->size && H->a[r].h < sv) { s = r; }
        if (s == pos) return;
        hcell t = H->a[s];
        H->a[s] = H->a[pos];
        H->a[pos] = t;
        pos = s;
    }
}

static void heap_insert(heap_t *H, const hcell *c)
{
    if (H->size == H->cap)
    {
        if (c->h < H->a[0].h) /* increase_key refuses a smaller value */
            return;
        H->a[0] = *c;
        heapify(H, 0);
        return;
    }
    H->a[H->size++] = *c;
    for (int i = (H->size - 1) / 2; i >= 0; i--)
        heapify(H, i);
}

static hcell heap_getmax(const heap_t *H)
{
    if (H->size <= 1)
        return H->a[0];
    hcell m = H->a[H->size - 1];
    for (int k = H->size - 2; k >= H->size / 2; k--)
        if (H->a[k].h > m.h)
            m = H->a[k];
    return m;
}

/* ---------------------------------------------------------------------- */
/* DSLIM_BinarySearch / BinFindMin / BinFindMax, dslim_query.cpp:854-994    */
/* ---------------------------------------------------------------------- */
static int bin_find_min(const orc_entry *e, float pm, int mn, int mx)
{
    for (;;)
    {
        int half = (mn + mx) / 2;
        if (mx - mn < 20)
        {
            int cur = mn;
            while (e[cur].mass < pm) cur++;
            return cur;
        }
        if (pm > e[half].mass) { mn = half; continue; }
        if (pm < e[half].mass) { mx = half; continue; }
        while (half >= 0 && pm == e[half].mass) half--;
        return half + 1;
    }
}

static int bin_find_max(const orc_entry *e, uint32_t n, float pm, int mn, int mx)
{
    for (;;)
    {
        int half = (mn + mx) / 2;
        if (mx - mn < 20)
        {
            int cur = mx;
            while (e[cur].mass > pm) cur--;
            return cur;
        }
        if (pm > e[half].mass) { mn = half; continue; }
        if (pm < e[half].mass) { mx = half; continue; }
        half++;
        while (half < (int)n && pm == e[half].mass) half++;
        return half - 1;
    }
}

static int binary_search(const orc_length *ix, float precmass, double dM, int *minl, int *maxl)
{
    const float pm1 = (float)((double)precmass - dM), pm2 = (float)((double)precmass + dM);
    const orc_entry *e = ix->entries;
    if (ix->n == 0)
        return 0;
    int mn = 0, mx = (int)ix->n - 1;
    if (dM < 0.0) { *minl = mn; *maxl = mx; return 0; }
    if (pm1 < e[mn].mass) *minl = mn;
    else if (pm1 > e[mx].mass) { *minl = mx; *maxl = mx; return 0; }
    else *minl = bin_find_min(e, pm1, mn, mx);
    if (pm2 > e[mx].mass) *maxl = mx;
    else if (pm2 < e[mn].mass) { *minl = mn; *maxl = mn; return 0; }
    else *maxl = bin_find_max(e, ix->n, pm2, mn, mx);
    return (e[*maxl].mass <= pm2 && e[*minl].mass >= pm1);
}

static inline uint32_t lower_bound_u32(const uint32_t *a, uint32_t lo, uint32_t hi, uint32_t v)
{
    while (lo < hi) { uint32_t m = lo + (hi - lo) / 2; if (a[m] < v) lo = m + 1; else hi = m; }
    return lo;
}
static inline uint32_t upper_bound_u32(const uint32_t *a, uint32_t lo, uint32_t hi, uint32_t v)
{
    while (lo < hi) { uint32_t m = lo + (hi - lo) / 2; if (a[m] <= v) lo = m + 1; else hi = m; }
    return lo;
}

/* ---------------------------------------------------------------------- */
/* expeRT::ModelTailFit(Results*), expeRT.cpp:572-718, with LinearFit       */
/* (1297-1345), rargmax/argmax/largmax (1208-1257)                          */
/* ---------------------------------------------------------------------- */
static void linear_fit(const double *x, const double *y, int n, double *a, double *b)
{
    if (n == 1) { *a = 0.0; *b = y[0]; return; }
    double xbar = 0.0, ybar = 0.0, top = 0.0, bot = 0.0;
    for (int i = 0; i < n; i++) { xbar = xbar + x[i]; ybar = ybar + y[i]; }
    xbar = xbar / (double)n;
    ybar = ybar / (double)n;
    for (int i = 0; i < n; i++)
    {
        top = top + (x[i] - xbar) * (y[i] - ybar);
        bot = bot + (x[i] - xbar) * (x[i] - xbar);
    }
    *a = top / bot;
    *b = ybar - *a * xbar;
}

void orc_tailfit(const double *yy, int cpsms, int hyp, int32_t *mu, int32_t *beta,
                 int32_t *stt1_out, int32_t *end1_out, uint32_t *flags)
{
    double mu_t = 0.0, beta_t = 4.0;
    /* A top hyperscore past the histogram (flagged ORC_FLAG_HIST_OOB) makes
     * the reference read survival[] beyond its 1002 bins (undefined): here,
     * as on the device, bins past the histogram hold 0 and the slice stops
     * at its last bin. */
    int end1 = hyp - 1;
    for (int q = (hyp - 1 < ORC_HIST_BINS - 1 ? hyp - 1 : ORC_HIST_BINS - 1); q >= 0; q--)
        if (yy[q] >= 1.0) { end1 = q; break; }
    int stt1 = 0;
    for (int q = 0; q <= end1 && q < ORC_HIST_BINS; q++)
        if (yy[q] >= 1.0) { stt1 = q; break; }
    if (stt1 == end1)
        end1 += 1;
    int n = end1 - stt1 + 1;
    if (n < 0) n = 0;
    if (stt1 + n > ORC_HIST_BINS) n = ORC_HIST_BINS - stt1;
    if (cpsms < 1)
    {
        mu_t = 0;
        beta_t = 100;
    }
    else if (n == 0)
    {
        /* empty slice: xbar = ybar = 0/0 */
        *flags |= ORC_FLAG_TAILFIT_EMPTY;
        mu_t = NAN;
        beta_t = NAN;
    }
    else
    {
        /* sx[-1] is read when mark == -1; one extra leading slot stands for it
         * and holds +0.0 (the reference reads the allocator's chunk header). */
        double sxbuf[ORC_HIST_BINS + 3];
        double *sx = sxbuf + 1;
        sxbuf[0] = 0.0;
        double c = 0.0;
        for (int i = 0; i < n; i++)
        {
            c = c + yy[stt1 + i];
            sx[i] = c;
        }
        for (int i = 0; i < n; i++) sx[i] /= (double)cpsms;
        for (int i = 0; i < n; i++) sx[i] += -1.0;
        for (int i = 0; i < n; i++) sx[i] = -sx[i];
        for (int i = 0; i < n; i++) if (sx[i] > 1.0) sx[i] = 0.999;
        int repl = n - 1;
        for (int q = n - 1; q >= 0; q--)
            if (sx[q] >= 1e-4) { repl = q; break; }
        const double rv = sx[repl];
        for (int i = 0; i < n; i++) if (sx[i] <= 0.0) sx[i] = rv;
        for (int i = 0; i < n; i++) sx[i] = log10(sx[i]);
        int mark = 0, mark2 = 0;
        const double hgt = sx[n - 1] - sx[0];
        if (n > 3)
        {
            const double t1 = sx[0] + hgt * 0.22, t2 = sx[0] + hgt * 0.87;
            int lm = 0;
            for (int q = 0; q <= n - 1; q++) if (sx[q] <= t1) { lm = q; break; }
            mark = lm - 1;
            mark2 = n - 1;
            for (int q = n - 1; q >= 0; q--) if (sx[q] >= t2) { mark2 = q; break; }
            if (mark2 == n) mark2 -= 1;
            if (mark >= mark2) mark = mark2 - 1;
        }
        else if (n == 3)
        {
            const double t1 = sx[0] + hgt * 0.22;
            int lm = 0;
            for (int q = 0; q <= n - 1; q++) if (sx[q] <= t1) { lm = q; break; }
            mark = lm - 1;
            mark2 = n - 1;
            if (mark >= mark2) mark = mark2 - 1;
        }
        else
        {
            mark = 0;
            mark2 = n - 1;
        }
        if (mark < 0)
            *flags |= ORC_FLAG_TAILFIT_OOB;
        const int m = mark2 - mark + 1;
        double X[ORC_HIST_BINS + 2];
        for (int i = 0; i < m; i++) X[i] = (double)(stt1 + mark + i);
        linear_fit(X, sx + mark, m, &mu_t, &beta_t);
    }
    *mu = x86_d2i(mu_t * 1e6);
    *beta = x86_d2i(beta_t * 1e6);
    *stt1_out = stt1;
    *end1_out = end1;
}

/* ---------------------------------------------------------------------- */
/* DSLIM_QuerySpectrum, dslim_query.cpp:515-842 (shared-memory mode)        */
/* ---------------------------------------------------------------------- */
typedef struct
{
    int16_t bc, yc;
    int64_t ibc, iyc;
} byc_t;

int orc_query(const orc_length *lens, uint32_t nlen, const orc_params *p,
              const uint32_t *qidx, const uint32_t *qmoz, const uint32_t *qint,
              const float *qprec, const double *dM_per_spec, uint32_t nspec, int tie_rule,
              orc_result *out, uint32_t *hist_out, int threads)
{
    /* lgfact, utils.h:115-131, extended past MAX_SHDPEAKS for defined
     * behaviour (those inputs are flagged) */
    static double lgfact[65536];
    static int lg_init = 0;
    if (!lg_init)
    {
        lgfact[0] = lgfact[1] = log10(1);
        for (int i = 2; i < 65536; i++) lgfact[i] = log10(i) + lgfact[i - 1];
        lg_init = 1;
    }
    uint32_t maxn = 1;
    for (uint32_t l = 0; l < nlen; l++) if (lens[l].n > maxn) maxn = lens[l].n;
    const uint32_t dF = p->dF, scale = p->scale;
    const double maxmass = p->max_mass;
    uint32_t num = p->topmatches == 0 ? 1 : p->topmatches;
    num = (uint32_t)(floor(log2((double)num) + 0.999));
    const int heapcap = (1 << num) - 1;
    if (heapcap > 64) return -1;
    if (threads <= 0) threads = 1;

#pragma omp parallel num_threads(threads)
    {
        byc_t *byc = (byc_t *)calloc(maxn, sizeof(byc_t));
        double *surv = (double *)calloc(ORC_HIST_BINS, sizeof(double));
#pragma omp for schedule(dynamic, 4)
        for (int64_t s = 0; s < (int64_t)nspec; s++)
        {
            const uint32_t *QA = qmoz + qidx[s], *IP = qint + qidx[s];
            const uint32_t qn = qidx[s + 1] - qidx[s];
            const double dM = dM_per_spec ? dM_per_spec[s] : p->dM;
            orc_result r;
            memset(&r, 0, sizeof(r));
            heap_t H;
            memset(&H, 0, sizeof(H));
            H.cap = heapcap;
            hcell best = {0.0f, -1, -1, 0, 0};
            uint32_t flags = 0, cpsms = 0;
            uint64_t bytes = 0;
            memset(surv, 0, sizeof(double) * ORC_HIST_BINS);

            for (uint32_t ixx = 0; ixx < nlen; ixx++)
            {
                const orc_length *ix = &lens[ixx];
                const uint32_t speclen = 2 * p->maxz * (ix->L - 1), half = speclen / 2;
                int minl = 0, maxl = 0;
                if (!binary_search(ix, qprec[s], dM, &minl, &maxl) || maxl < minl)
                    continue;
                for (uint32_t k = 0; k < qn; k++)
                {
                    const uint32_t qion = QA[k], intn = IP[k];
                    if (!((double)qion > dF && (double)qion < ((maxmass * scale) - 1 - dF)))
                        continue;
                    bytes += 4ull * (2 * dF + 2);
                    for (uint32_t bin = qion - dF; bin < qion + 1 + dF; bin++)
                    {
                        const uint32_t st = ix->bA[bin], en = ix->bA[bin + 1];
                        if (en - st < 1) continue;
                        const uint32_t stt = lower_bound_u32(ix->iA, st, en, (uint32_t)minl * speclen);
                        const uint32_t ends1 = upper_bound_u32(ix->iA, stt, en,
                                                               ((uint32_t)(maxl + 1) * speclen) - 1);
                        bytes += 4ull * (ends1 - stt);
                        for (uint32_t ion = stt; ion < ends1; ion++)
                        {
                            const uint32_t raw = ix->iA[ion];
                            const int ppid = (int)(raw / speclen);
                            const int isY = (int)((raw % speclen) / half), isB = 1 - isY;
                            byc_t *el = &byc[ppid];
                            el->bc = (int16_t)(el->bc + isB);
                            el->ibc += (int64_t)(uint32_t)(intn * (uint32_t)isB);
                            el->yc = (int16_t)(el->yc + isY);
                            el->iyc += (int64_t)(uint32_t)(intn * (uint32_t)isY);
                        }
                    }
                }
                for (int it = minl; it <= maxl; it++)
                {
                    const uint16_t bcc = (uint16_t)byc[it].bc, ycc = (uint16_t)byc[it].yc;
                    const uint16_t shpk = (uint16_t)(bcc + ycc);
                    if (shpk >= p->min_shp)
                    {
                        if (bcc >= ORC_MAXSHP || ycc >= ORC_MAXSHP)
                            flags |= ORC_FLAG_LGFACT_OOB;
                        const double h1 = lgfact[bcc] + lgfact[ycc];
                        const float h = (float)(h1 + log10((double)(1 + byc[it].ibc)) +
                                                log10((double)(1 + byc[it].iyc)) - 6);
                        if (h > 0)
                        {
                            hcell c = {h, (int32_t)ixx, it, shpk, (uint16_t)speclen};
                            heap_insert(&H, &c);
                            cpsms += 1;
                            const float h10 = h * 10.0f;
                            int bin = (int)((double)h10 + 0.5);
                            if (bin >= ORC_HIST_BINS) { flags |= ORC_FLAG_HIST_OOB; bin = ORC_HIST_BINS - 1; }
                            surv[bin] += 1;
                            if (h > best.h) best = c; /* strict: keeps the lowest (ixx, psid) */
                        }
                    }
                }
                memset(byc + minl, 0, sizeof(byc_t) * (size_t)(maxl - minl + 1));
            }

            r.cpsms = cpsms;
            r.post_bytes = bytes;
            hcell top = tie_rule == 0 ? heap_getmax(&H) : best;
            if (cpsms == 0) { top.ixx = -1; top.psid = -1; top.h = 0; top.shp = 0; top.tot = 0; }
            r.idxoffset = top.ixx;
            r.psid = top.psid;
            r.sharedions = top.shp;
            r.totalions = top.tot;
            r.hyperscore = top.h;
            if (cpsms >= p->min_cpsm)
            {
                /* maxhypscore = (h*10 + 0.5) with a float product (dslim_query.cpp:778) */
                const hcell hm = heap_getmax(&H);
                const float h10 = hm.h * 10.0f;
                const int maxhyp = x86_d2i((double)h10 + 0.5);
                int32_t mu, beta, s1, e1;
                orc_tailfit(surv, (int)cpsms, maxhyp, &mu, &beta, &s1, &e1, &flags);
                double w = mu, b = beta;
                w /= 1e6;
                b /= 1e6;
                const double lgs = (w * maxhyp) + b;
                double e_x = pow(10, lgs);
                e_x *= cpsms;
                r.mu = mu;
                r.beta = beta;
                r.minhyp = s1;
                r.nexthyp = e1;
                r.maxhyp = maxhyp;
                r.evalue = e_x;
                r.reported = e_x < p->expect_max;
            }
            r.flags = flags;
            out[s] = r;
            if (hist_out)
                for (int b = 0; b < ORC_HIST_BINS; b++)
                    hist_out[(size_t)s * ORC_HIST_BINS + b] = (uint32_t)surv[b];
        }
        free(byc);
        free(surv);
    }
    return 0;
}
