// Host-side preparation for the DSLIM path: ion-key tables, the lgfact
// table, database-entry enumeration (base peptides + variable-mod variants)
// and the division constants used by the query kernel.
//
// Compiled with -ffp-contract=off: the tables are derived with the same
// double arithmetic the reference uses, and must round the same way on
// x86-64 and aarch64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

#include "hc_internal.h"

namespace hc {

namespace {

// Residue masses and the static carbamidomethyl-C mod (utils.cpp:41-98),
// single precision as in the reference.
constexpr float kNaa = -20000.0f;
const float kAAMass[26] = {
    71.03712f, kNaa, 103.00919f, 115.030f, 129.0426f, 147.068f, 57.02146f, 137.060f,
    113.084f,  kNaa, 128.094f,   113.084f, 131.0405f, 114.043f, kNaa,      97.0527f,
    128.05858f, 156.1012f, 87.032f, 101.0476f, kNaa, 99.06841f, 186.0793f, kNaa,
    163.0633f, kNaa};
const float kStatMods[26] = {0, 0, 57.021464f, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                             0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
constexpr float kH2O = 18.015f;
constexpr double kProton = 1.00727647;

// GETAA(x, z) (utils.cpp:101): float residue + float static mod, then the
// proton mass times z added in double.
inline double getaa(int a, double z)
{
    float s = kAAMass[a] + kStatMods[a];
    return (double)s + kProton * z;
}

float pep_mass(const uint8_t *seq, uint32_t L)
{
    // UTILS_CalculatePepMass (utils.cpp:290-303): two float additions per residue
    float m = kH2O;
    for (uint32_t l = 0; l < L; l++)
    {
        m += kAAMass[seq[l] - 'A'];
        m += kStatMods[seq[l] - 'A'];
    }
    return m;
}

float mod_mass(const hc_params &p, const uint8_t *seq, uint32_t L, uint32_t modnum)
{
    // UTILS_CalculateModMass (utils.cpp:337-362): its loop advances `start`
    // by a shift of 4 but then shifts the masked value right by `start`
    // itself; the hardware takes that count mod 32, the result is 0, so
    // only the first mod's scaled mass (as float / scale) is added.
    float m = pep_mass(seq, L);
    uint32_t first = modnum & 0xF;
    if (first != 0)
        m += (float)p.mod_mass[first - 1] / (float)p.scale;
    return m;
}

struct VariantGen
{
    const hc_params *p;
    int cond_of[26];
    int nterm = -1;  // mod condition of the N-terminus ('^'), -1 if none
    const uint8_t *seq;
    uint32_t L, seqid;
    hc_entry *out;
    int64_t n, cap;

    // Depth-first enumeration of MODS_ModList (mods.cpp:333-384): at each
    // position first the branch that modifies it, then the one that does
    // not; an entry is emitted on entering a position right after a new mod.
    // Positions are virtual: v = 0 is the N-terminus (modifiable only by a
    // '^' mod, an extension; site bit kNtermBit), v >= 1 is residue v-1.
    void walk(int *conds, int total, uint64_t sites, uint32_t modnum, int v, bool novel, int seen)
    {
        if (novel)
        {
            if (n < cap && out)
            {
                hc_entry &e = out[n];
                e.seqid = seqid;
                e.sites = sites;
                e.modnum = modnum;
                e.pad = 0;
                e.mass = mod_mass(*p, seq, L, modnum);
            }
            n++;
        }
        if (total == 0 || v > (int)L)
            return;
        const int c = v == 0 ? nterm : cond_of[seq[v - 1] - 'A'];
        const int bit = v == 0 ? kNtermBit : v - 1;
        if (c != -1 && conds[c] > 0)
        {
            conds[c] -= 1;
            walk(conds, total - 1, sites | (1ull << bit),
                 modnum + (uint32_t)((1u << (4 * seen)) * (uint32_t)(1 + c)), v + 1, true, seen + 1);
            conds[c] += 1;
        }
        walk(conds, total, sites, modnum, v + 1, false, seen);
    }
};

}  // namespace

void make_enum_const(const hc_params &p, EnumConst *e)
{
    std::memset(e, 0, sizeof(*e));
    for (int a = 0; a < 26; a++)
    {
        e->aa[a] = kAAMass[a];
        e->stat[a] = kStatMods[a];
        e->cond_of[a] = -1;
    }
    e->nterm = -1;
    e->h2o = kH2O;
    const uint32_t nm = p.nmods < HC_MAX_MODS ? p.nmods : HC_MAX_MODS;
    for (uint32_t m = 0; m < nm; m++)
    {
        for (int j = 0; j < 4 && p.mod_res[m][j]; j++)
        {
            const int c = p.mod_res[m][j] - 'A';
            if (p.mod_res[m][j] == '^') e->nterm = (int8_t)m;
            else if (c >= 0 && c < 26) e->cond_of[c] = (int8_t)m;
        }
        e->limit[m] = p.mod_per_pep[m];
        e->modadd[m] = (float)p.mod_mass[m] / (float)p.scale;
    }
    e->nmods = nm;
    e->vmods = p.vmods_per_pep;
}

void make_ion_tables(const hc_params &p, IonTables *t)
{
    std::memset(t, 0, sizeof(*t));
    const double scale = p.scale;
    for (int a = 0; a < 26; a++)
    {
        for (uint32_t z = 0; z < p.maxz && z < (uint32_t)kMaxZ; z++)
        {
            // UTILS_GenerateSpectrum, utils.cpp:257-270
            t->bf[a][z] = (uint32_t)((getaa(a, z + 1) * scale) / (z + 1));
            t->yf[a][z] = (uint32_t)(((getaa(a, z + 1) + kH2O) * scale) / (z + 1));
            t->inc[a][z] = (uint32_t)((getaa(a, 0) * scale) / (z + 1));
            // UTILS_GenerateModSpectrum, utils.cpp:441-454 (division comes later)
            t->bfm[a][z] = (uint32_t)(getaa(a, z + 1) * scale);
            t->yfm[a][z] = (uint32_t)((getaa(a, z + 1) + kH2O) * scale);
        }
        t->incm[a] = (uint32_t)(getaa(a, 0) * scale);
    }
    for (uint32_t m = 0; m < p.nmods && m < 16; m++)
        t->mod_mass[m] = p.mod_mass[m];
    t->maxz = p.maxz;
    t->scale = p.scale;
    t->min_mass = p.min_mass;
    t->max_mass = p.max_mass;
}

// The y1 keys, charges 0 .. maxz-1, of the entries with entry-class code
// `code` (hc_index.cu, entry_code): the first y ion of k_ion_keys's loop,
// i.e. utils.cpp:257-270 without mods and utils.cpp:441-500 with them (the
// undivided sum plus the mod at the last residue, then integer division by
// the charge); illegal masses give zero keys.
void class_keys_of(const hc_params &p, const IonTables &t, uint32_t code, uint32_t *keys)
{
    const uint32_t top = p.max_mass * p.scale;
    const bool illegal = code == kCodes - 1;
    for (uint32_t z = 0; z < p.maxz && z < (uint32_t)kMaxZ; z++)
    {
        uint32_t v;
        if (illegal) v = 0;
        else if (!(code & 0x200u)) v = code < 26 ? t.yf[code][z] : 0u;
        else
        {
            const uint32_t r = (code >> 4) & 0x1Fu, qy = code & 0xFu;
            v = r < 26 ? (t.yfm[r][z] + (qy ? t.mod_mass[qy - 1] : 0u)) / (z + 1) : 0u;
        }
        keys[z] = (!illegal && v >= top) ? top - 1 : v;
    }
}

void make_query_const(QueryConst *q)
{
    // hcp::utils::lgfact (utils.h:115-131): val[0] = val[1] = log10(1),
    // val[i] = log10(i) + val[i-1]. Entries past 80 exist only so that the
    // device never reads out of bounds; results using them are flagged.
    q->lgfact[0] = q->lgfact[1] = std::log10(1.0);
    for (int i = 2; i < kLgTable; i++)
        q->lgfact[i] = std::log10((double)i) + q->lgfact[i - 1];
    for (int i = 0; i < kLgTable; i++)
        q->lgfact_f[i] = (float)q->lgfact[i];
    q->log10_tab = nullptr;
}

void make_log10_table(double *t, uint32_t n)
{
    // log10(n) for the integers the hyperscore takes logarithms of
    // (log10(1 + ibc), dslim_query.cpp:698), from the host's libm: the same
    // function the reference calls. Filled by all host threads.
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nt; k++)
        th.emplace_back([=]() {
            for (uint32_t i = k; i < n; i += nt) t[i] = std::log10((double)i);
        });
    for (auto &x : th) x.join();
}

int64_t make_entries(const hc_params &p, uint32_t L, const uint8_t *seqs, uint32_t npep,
                     hc_entry *out, int64_t cap)
{
    // LBE_GeneratePeps (lbe_internal.cpp:204-229): one entry per peptide, in
    // file order; then the variants of MODS_GenerateMods (mods.cpp:448-496),
    // peptide by peptide.
    VariantGen g{};
    g.p = &p;
    g.L = L;
    g.out = out;
    g.cap = cap;
    for (int i = 0; i < 26; i++) g.cond_of[i] = -1;
    for (uint32_t m = 0; m < p.nmods && m < HC_MAX_MODS; m++)
        for (int j = 0; j < 4 && p.mod_res[m][j]; j++)
        {
            int c = p.mod_res[m][j] - 'A';
            if (p.mod_res[m][j] == '^') g.nterm = (int)m;
            else if (c >= 0 && c < 26) g.cond_of[c] = (int)m;
        }
    for (uint32_t i = 0; i < npep; i++)
    {
        if (out && g.n < cap)
        {
            hc_entry &e = out[g.n];
            e.mass = pep_mass(seqs + (size_t)i * L, L);
            e.seqid = i;
            e.sites = 0;
            e.modnum = 0;
            e.pad = 0;
        }
        g.n++;
    }
    if (p.vmods_per_pep > 0 && p.nmods > 0)
    {
        int conds[HC_MAX_MODS] = {0};
        for (uint32_t m = 0; m < p.nmods && m < HC_MAX_MODS; m++) conds[m] = (int)p.mod_per_pep[m];
        for (uint32_t i = 0; i < npep; i++)
        {
            g.seq = seqs + (size_t)i * L;
            g.seqid = i;
            g.walk(conds, (int)p.vmods_per_pep, 0, 0, 0, false, 0);
        }
    }
    return g.n;
}

void division_magic(uint32_t d, uint32_t *magic, uint32_t *sh)
{
    // Granlund & Montgomery, "Division by Invariant Integers using
    // Multiplication" (PLDI 1994), Thm 4.2 with N = 31-bit dividends:
    // l = ceil(log2 d), m = ceil(2^(31+l) / d) < 2^32, and
    // floor(x/d) = floor(m*x / 2^(31+l)) = umulhi(x, m) >> (l-1).
    uint32_t l = 0;
    while ((1ull << l) < d) l++;
    if (l == 0)
    {   // d == 1: umulhi(x, 2^31) = x >> 1, so use l = 1 and m = 2^32 - 1? keep exact:
        *magic = 0xFFFFFFFFu;  // not used: speclen >= 2 always
        *sh = 0;
        return;
    }
    const unsigned __int128 num = (unsigned __int128)1 << (31 + l);
    const uint64_t m = (uint64_t)((num + d - 1) / d);
    *magic = (uint32_t)m;
    *sh = l - 1;
}

}  // namespace hc
