// Device construction of the SLM index of one peptide length
// (DSLIM_Construct, source/core/dslim.cpp:46-138):
//   0. entries (base peptides, then their variable-mod variants) enumerated
//      on the device (LBE_GeneratePeps, lbe_internal.cpp:204-229, and
//      MODS_GenerateMods, mods.cpp:448-496),
//   1. entries sorted by mass on the device (stable LSD radix sort; the
//      reference uses std::sort, lbe_internal.cpp:184-187),
//   2. ion keys of every entry from integer tables (UTILS_GenerateSpectrum /
//      UTILS_GenerateModSpectrum, utils.cpp:231-505, with the legality rules
//      of DSLIM_ConstructChunk, dslim.cpp:296-323),
//   3. postings iA = ion ids stably sorted by key (the reference's key/value
//      quicksort + per-bucket sort, dslim.cpp:361-388 and 452-482, leave ids
//      ascending inside every bucket: a stable sort gives exactly that),
//   4. bucket offsets bA from the sorted keys (the exclusive scan of
//      dslim.cpp:97-125).
#include <cstdio>

#include <algorithm>
#include <vector>

#include "hc_internal.h"

namespace hc {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;  // 4096 items per CTA
constexpr int kRadix = 256;
constexpr int kRsWarps = kRsThreads / 32;

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- stable LSD radix sort, 8-bit digits ----------------------------------

__global__ void k_rs_upsweep(const uint32_t *__restrict__ keys, size_t n, int shift,
                             uint32_t *__restrict__ tile_hist, uint32_t ntiles)
{
    __shared__ uint32_t h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kRsTile;
#pragma unroll 4
    for (int i = 0; i < kRsItems; i++)
    {
        size_t idx = base + (size_t)i * kRsThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
        tile_hist[(size_t)d * ntiles + blockIdx.x] = h[d];
}

// Stable ranking: warp w owns items [w*512, w*512+512) of the tile in order;
// inside a round of 32 items, lanes with equal digits are ranked by lane id
// (match.any + lanemask_lt), rounds advance a per-warp digit counter, and the
// warps' counters are scanned per digit.
__global__ void k_rs_downsweep(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                               uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
                               size_t n, int shift, const uint32_t *__restrict__ tile_off,
                               uint32_t ntiles, int write_keys)
{
    __shared__ uint32_t whist[kRsWarps][kRadix];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kRsWarps * kRadix; i += blockDim.x) (&whist[0][0])[i] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kRsTile + (size_t)warp * (kRsItems * 32);
    uint32_t k[kRsItems], v[kRsItems], rank[kRsItems];
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kRsItems; r++)
    {
        const size_t idx = base + (size_t)r * 32 + lane;
        const bool ok = idx < n;
        k[r] = ok ? keys_in[idx] : 0u;
        v[r] = ok ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
        const uint32_t d = ok ? ((k[r] >> shift) & 0xFF) : 0x100u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t before = (d < kRadix) ? whist[warp][d] : 0u;
        rank[r] = before + __popc(peers & lt);
        __syncwarp();
        if (d < kRadix && (peers >> lane) == 1u)  // highest lane of the group
            whist[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
    {
        uint32_t run = tile_off[(size_t)d * ntiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kRsWarps; w++)
        {
            uint32_t c = whist[w][d];
            whist[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRsItems; r++)
    {
        const size_t idx = base + (size_t)r * 32 + lane;
        if (idx < n)
        {
            const uint32_t d = (k[r] >> shift) & 0xFF;
            const uint32_t dst = whist[warp][d] + rank[r];
            if (write_keys) keys_out[dst] = k[r];
            vals_out[dst] = v[r];
        }
    }
}

// ---- exclusive scan of u32 (in place), recursive over block sums ----------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tiles(uint32_t *__restrict__ a, size_t n, uint32_t *__restrict__ sums)
{
    __shared__ uint32_t wsum[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t x[kScanItems], t = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
    {
        x[i] = (base + i < n) ? a[base + i] : 0u;
        uint32_t c = x[i];
        x[i] = t;
        t += c;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t s = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
        if (lane >= o) s += y;
    }
    if (lane == 31) wsum[warp] = s;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = s - t + (warp ? wsum[warp - 1] : 0u);
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) a[base + i] = x[i] + excl;
    if (threadIdx.x == kScanThreads - 1 && sums) sums[blockIdx.x] = excl + t;
}

__global__ void k_scan_add(uint32_t *__restrict__ a, size_t n, const uint32_t *__restrict__ sums)
{
    const uint32_t off = sums[blockIdx.x];
    const size_t base = (size_t)blockIdx.x * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
        if (base + i < n) a[base + i] += off;
}

cudaError_t scan_exclusive(uint32_t *a, size_t n, uint32_t *tmp, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const size_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1)
    {
        k_scan_tiles<<<1, kScanThreads, 0, st>>>(a, n, nullptr);
        return cudaGetLastError();
    }
    k_scan_tiles<<<(unsigned)nb, kScanThreads, 0, st>>>(a, n, tmp);
    cudaError_t e = scan_exclusive(tmp, nb, tmp + nb, st);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)nb, 256, 0, st>>>(a, n, tmp);
    return cudaGetLastError();
}

size_t scan_tmp_words(size_t n)
{
    size_t t = 0;
    while (n > (size_t)kScanTile)
    {
        n = (n + kScanTile - 1) / kScanTile;
        t += n;
    }
    return t + 16;
}

// Sorts (keys, vals) by the low `bits` bits of the keys, stably. Ping-pongs
// between the given buffers (all four must be valid, n words each); returns
// which pair holds the result (0 or 1). With positions_as_values the input
// values are not read: value i is the input position i.
cudaError_t radix_sort(uint32_t *keys0, uint32_t *keys1, uint32_t *vals0, uint32_t *vals1, size_t n,
                       int bits, uint32_t *hist, uint32_t *scan_tmp, cudaStream_t st, int *which,
                       int *launches, bool keys_out, bool positions_as_values)
{
    const uint32_t ntiles = (uint32_t)((n + kRsTile - 1) / kRsTile);
    int cur = 0;
    const uint32_t *vin = positions_as_values ? nullptr : vals0;
    for (int shift = 0; shift < bits; shift += 8)
    {
        uint32_t *kin = cur ? keys1 : keys0, *kout = cur ? keys0 : keys1;
        uint32_t *vout = cur ? vals0 : vals1;
        if (n)
        {
            k_rs_upsweep<<<ntiles, kRsThreads, 0, st>>>(kin, n, shift, hist, ntiles);
            cudaError_t e = scan_exclusive(hist, (size_t)ntiles * kRadix, scan_tmp, st);
            if (e != cudaSuccess) return e;
            const int last = shift + 8 >= bits;
            k_rs_downsweep<<<ntiles, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, hist,
                                                          ntiles, (last && !keys_out) ? 0 : 1);
            *launches += 3;
        }
        vin = vout;
        cur ^= 1;
    }
    *which = cur;
    return cudaGetLastError();
}

// ---- entries ---------------------------------------------------------------

// Entry enumeration on the device, one thread per peptide. The base entry of
// peptide i (LBE_GeneratePeps, lbe_internal.cpp:204-229) is entry i; its
// variable-mod variants (MODS_GenerateMods, mods.cpp:448-496) follow all base
// entries, peptide by peptide, in the order of MODS_ModList's depth-first walk
// (mods.cpp:333-384): at each modifiable position the branch that modifies it
// comes before the one that skips it, and a variant is emitted as each mod is
// added. Here the walk is a loop over a stack of chosen positions. The first
// pass (out == nullptr) counts the variants per peptide; the second writes
// them at npep + voff[i].
__global__ void k_enum_entries(const uint8_t *__restrict__ seqs, uint32_t L, uint32_t npep, EnumConst ec,
                               const uint32_t *__restrict__ voff, uint32_t *__restrict__ vcount,
                               float *__restrict__ mass, uint32_t *__restrict__ seqid,
                               uint64_t *__restrict__ sites, uint32_t *__restrict__ modnum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npep) return;
    const uint8_t *s = seqs + (size_t)i * L;
    // UTILS_CalculatePepMass: two float additions per residue, in order
    float pm = ec.h2o;
    for (uint32_t l = 0; l < L; l++)
    {
        pm += ec.aa[s[l] - 'A'];
        pm += ec.stat[s[l] - 'A'];
    }
    const bool write = voff != nullptr;
    if (write)
    {
        mass[i] = pm;
        seqid[i] = i;
        sites[i] = 0;
        modnum[i] = 0;
    }
    uint32_t k = 0;
    if (ec.vmods > 0 && ec.nmods > 0)
    {
        int cap[HC_MAX_MODS];
        for (int m = 0; m < HC_MAX_MODS; m++) cap[m] = (int)ec.limit[m];
        uint8_t pos[64];
        uint32_t d = 0, mn = 0;
        uint64_t st = 0;
        uint32_t start = 0;
        const uint64_t at = write ? (uint64_t)npep + voff[i] : 0;
        for (;;)
        {
            // virtual positions: q = 0 is the N-terminus (a '^' mod, an
            // extension; site bit kNtermBit), q >= 1 is residue q - 1
            int p = -1;
            if (d < ec.vmods && d < 64)
                for (uint32_t q = start; q <= L; q++)
                {
                    const int c = q == 0 ? ec.nterm : ec.cond_of[s[q - 1] - 'A'];
                    if (c >= 0 && cap[c] > 0)
                    {
                        p = (int)q;
                        break;
                    }
                }
            if (p >= 0)
            {
                const int c = p == 0 ? ec.nterm : ec.cond_of[s[p - 1] - 'A'];
                cap[c] -= 1;
                pos[d] = (uint8_t)p;
                mn += (1u << ((4u * d) & 31u)) * (uint32_t)(1 + c);  // shift count taken mod 32, as the CPU does
                st |= 1ull << (p == 0 ? kNtermBit : p - 1);
                d++;
                if (write)
                {
                    // UTILS_CalculateModMass: only the first mod's mass is added
                    const uint64_t e = at + k;
                    mass[e] = pm + ec.modadd[(mn & 0xF) - 1];
                    seqid[e] = i;
                    sites[e] = st;
                    modnum[e] = mn;
                }
                k++;
                start = (uint32_t)p + 1;
            }
            else
            {
                if (d == 0) break;
                d--;
                const uint32_t q = pos[d];
                const int c = q == 0 ? ec.nterm : ec.cond_of[s[q - 1] - 'A'];
                cap[c] += 1;
                mn -= (1u << ((4u * d) & 31u)) * (uint32_t)(1 + c);
                st &= ~(1ull << (q == 0 ? kNtermBit : q - 1));
                start = q + 1;
            }
        }
    }
    if (!write) vcount[i] = k;
}

__global__ void k_mass_keys(const float *__restrict__ mass, uint32_t n, uint32_t *__restrict__ keys)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        uint32_t b = __float_as_uint(mass[i]);
        keys[i] = (b & 0x80000000u) ? ~b : (b | 0x80000000u);  // total order of floats
    }
}

__global__ void k_gather_entries(const uint32_t *__restrict__ perm, uint32_t n, const float *mass_in,
                                 const uint32_t *seqid_in, const uint64_t *sites_in,
                                 const uint32_t *modnum_in, float *mass, uint32_t *seqid,
                                 uint64_t *sites, uint32_t *modnum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const uint32_t j = perm[i];
        mass[i] = mass_in[j];
        seqid[i] = seqid_in[j];
        sites[i] = sites_in[j];
        modnum[i] = modnum_in[j];
    }
}

// ---- ion keys ----------------------------------------------------------------
// One thread per (entry, series, charge): writes the L-1 keys of one b or y
// series. Layout per entry: [b z=1][b z=2]..[y z=1][y z=2].., each L-1 long
// (utils.cpp:251-252).
__global__ void k_ion_keys(const IonTables *__restrict__ gt, uint32_t L, uint32_t n,
                           const float *__restrict__ mass, const uint32_t *__restrict__ seqid,
                           const uint64_t *__restrict__ sites, const uint32_t *__restrict__ modnum,
                           const uint8_t *__restrict__ seqs, uint32_t *__restrict__ keys,
                           uint32_t *__restrict__ nuninit)
{
    __shared__ IonTables t;
    for (int i = threadIdx.x; i < (int)(sizeof(IonTables) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t *>(&t)[i] = reinterpret_cast<const uint32_t *>(gt)[i];
    __syncthreads();
    const uint32_t maxz = t.maxz, nser = 2 * maxz;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)n * nser) return;
    const uint32_t k = (uint32_t)(gid / nser), s = (uint32_t)(gid % nser);
    const bool isY = s >= maxz;
    const uint32_t z = isY ? s - maxz : s;
    const uint32_t Lm1 = L - 1, speclen = nser * Lm1;
    uint32_t *out = keys + (size_t)k * speclen + (isY ? maxz * Lm1 : 0) + z * Lm1;
    const uint8_t *seq = seqs + (size_t)seqid[k] * L;
    const double m = mass[k];
    const double minm = t.min_mass, maxm = t.max_mass;
    const uint32_t top = t.max_mass * t.scale;
    const uint32_t mn = modnum[k];
    bool legal = (m >= minm && m <= maxm);
    if (mn != 0 && legal && !(m > minm && m < maxm))
    {   // mass exactly on a bound: the reference reads an uninitialised spectrum
        if (s == 0) atomicAdd(nuninit, 1u);
        legal = false;
    }
    if (!legal)
    {
        for (uint32_t l = 0; l < Lm1; l++) out[l] = 0;
        return;
    }
    if (mn == 0)
    {
        uint32_t v = isY ? t.yf[seq[L - 1] - 'A'][z] : t.bf[seq[0] - 'A'][z];
        out[0] = v >= top ? top - 1 : v;
        for (uint32_t l = 1; l < Lm1; l++)
        {
            const uint8_t a = isY ? seq[L - 1 - l] : seq[l];
            v += t.inc[a - 'A'][z];
            out[l] = v >= top ? top - 1 : v;
        }
        return;
    }
    // variable mods (utils.cpp:407-500): undivided running sums, plus the
    // masses of the first `counter` mods (b) or last `counter` mods (y),
    // then integer division by the charge
    uint32_t mods[16];
    int seen = 0;
    {
        uint32_t bm = mn;
        for (int i = 0; i < 8; i++)
        {
            int q = (int)(bm & 0xF) - 1;
            bm >>= 4;
            if (q != -1) mods[seen++] = t.mod_mass[q & 15];
        }
    }
    const uint64_t st = sites[k];
    uint32_t v = isY ? t.yfm[seq[L - 1] - 'A'][z] : t.bfm[seq[0] - 'A'][z];
    uint32_t madd = 0;
    int cnt = 0;
    // an N-terminal mod (extension) is the first mod and part of every b ion
    if (!isY && ((st >> kNtermBit) & 1ull) && seen > 0)
    {
        madd = mods[0];
        cnt = 1;
    }
    for (uint32_t l = 0; l < Lm1; l++)
    {
        const uint32_t pos = isY ? (L - 1 - l) : l;
        if (l > 0) v += t.incm[seq[pos] - 'A'];
        if (((st >> pos) & 1ull) && cnt < seen)
        {
            madd += isY ? mods[seen - 1 - cnt] : mods[cnt];
            cnt++;
        }
        uint32_t o = (v + madd) / (z + 1);
        out[l] = o >= top ? top - 1 : o;
    }
}

// bA[b] = first position of the sorted keys whose key is >= b, b in [0, nb]
// (the exclusive scan of the bucket counts, dslim.cpp:97-125): one thread per
// bucket, a lower bound over the keys. Neighbouring buckets search the same
// stretch of keys, so the probes share cache lines.
__global__ void k_bucket_bounds(const uint32_t *__restrict__ skeys, size_t M, uint32_t nb,
                                uint32_t *__restrict__ bA)
{
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= nb;
         b += (uint64_t)gridDim.x * blockDim.x)
    {
        size_t lo = 0, hi = M;
        while (lo < hi)
        {
            const size_t m = lo + ((hi - lo) >> 1);
            if (__ldg(skeys + m) < (uint32_t)b) lo = m + 1;
            else hi = m;
        }
        bA[b] = (uint32_t)lo;
    }
}

// Row table over the query postings: rows[b * stride + k] = first position in
// bucket b whose entry is >= k * kRowG (a lower bound on k * kRowG << 3).
// Column 0 is qA[b], column stride-1 is qA[b+1] (padding decodes past every
// entry, so it never precedes a lower bound).
__global__ void k_row_table(const uint32_t *__restrict__ qA, const uint32_t *__restrict__ qp, uint32_t nb,
                            uint32_t stride, uint32_t n, uint32_t *__restrict__ rows)
{
    const uint64_t total = (uint64_t)nb * stride;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t b = (uint32_t)(t / stride), k = (uint32_t)(t - (uint64_t)b * stride);
        uint32_t lo = __ldg(qA + b), hi = __ldg(qA + b + 1);
        if (k == stride - 1) lo = hi;
        else if (k > 0)
        {
            const uint32_t v = min(k * kRowG, n) << kQpEntryShift;
            while (lo < hi)
            {
                const uint32_t m = lo + ((hi - lo) >> 1);
                if (__ldg(qp + m) < v) lo = m + 1;
                else hi = m;
            }
        }
        rows[t] = lo;
    }
}

// padded bucket sizes: ceil4(bA[b+1] - bA[b]); entry nb is 0 (the scan makes it the total)
__global__ void k_pad_counts(const uint32_t *__restrict__ bA, uint32_t nb, uint32_t *__restrict__ pc)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b <= nb; b += gridDim.x * blockDim.x)
        pc[b] = b < nb ? ((bA[b + 1] - bA[b] + 3u) & ~3u) : 0u;
}

// ids (entry*speclen + ion, bucket order) -> query postings and their ions, one thread per bucket
__global__ void k_qpost(const uint32_t *__restrict__ bA, const uint32_t *__restrict__ ids,
                        const uint32_t *__restrict__ qA, uint32_t nb, uint32_t speclen, uint32_t half,
                        uint32_t *__restrict__ qp, uint16_t *__restrict__ qion)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    {
        const uint32_t s = bA[b], e = bA[b + 1], q = qA[b];
        for (uint32_t i = s; i < e; i++)
        {
            const uint32_t id = ids[i], entry = id / speclen, ion = id - entry * speclen;
            qp[q + (i - s)] = (entry << kQpEntryShift) | ((ion >= half ? 1u : 0u) << 2);
            qion[q + (i - s)] = (uint16_t)ion;
        }
    }
}

// counts query-posting words that are neither padding nor an (entry < n, ion < speclen)
// pair whose b/y bit matches its ion
__global__ void k_check_qpost(const uint32_t *__restrict__ qp, const uint16_t *__restrict__ qion, size_t total,
                              uint32_t n, uint32_t speclen, uint32_t half, uint32_t *__restrict__ bad)
{
    uint32_t b = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    {
        const uint32_t x = qp[i];
        if (x == kQpostPad) continue;
        const uint32_t ion = qion[i];
        if ((x & 3u) || (x >> kQpEntryShift) >= n || ion >= speclen || ((x >> 2) & 1u) != (ion >= half ? 1u : 0u)) b++;
    }
    if (b) atomicAdd(bad, b);
}

// query postings -> ids (the reference's iA), one thread per bucket
__global__ void k_qpost_ids(const uint32_t *__restrict__ bA, const uint32_t *__restrict__ qA,
                            const uint32_t *__restrict__ qp, const uint16_t *__restrict__ qion, uint32_t nb,
                            uint32_t speclen, uint32_t *__restrict__ ids)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
    {
        const uint32_t s = bA[b], e = bA[b + 1], q = qA[b];
        for (uint32_t i = s; i < e; i++)
            ids[i] = (qp[q + (i - s)] >> kQpEntryShift) * speclen + qion[q + (i - s)];
    }
}

// ---- entry classes and the search postings ------------------------------------
// (see ClassKeys in hc_internal.h)

// The class code of one entry: the facts k_ion_keys reads for the first y
// ion (legal mass, mod path, last residue, the mod there); kCodes - 1 for an
// illegal mass, and for a residue byte outside 'A'..'Z' a code no entry's
// postings can match (the build check then leaves it unclassed).
__device__ __forceinline__ uint32_t entry_code(double minm, double maxm, uint32_t L, const uint8_t *seq, double m,
                                               uint32_t mn, uint64_t st)
{
    bool legal = (m >= minm && m <= maxm);
    if (mn != 0 && legal && !(m > minm && m < maxm)) legal = false;
    if (!legal) return kCodes - 1;
    const uint32_t rl = (uint32_t)seq[L - 1] - 'A';
    if (rl >= 26u) return kCodes - 2;
    if (mn == 0) return rl;
    // the last mod, when the last residue carries one (utils.cpp:480-500)
    uint32_t last = 0;
    for (int i = 0; i < 8; i++)
    {
        const uint32_t q = (mn >> (4 * i)) & 0xFu;
        if (q) last = q;
    }
    const uint32_t qy = ((st >> (L - 1)) & 1ull) ? last : 0u;
    return 0x200u | (rl << 4) | qy;
}

__global__ void k_entry_codes(double minm, double maxm, uint32_t L, uint32_t n, const float *__restrict__ mass,
                              const uint32_t *__restrict__ seqid, const uint64_t *__restrict__ sites,
                              const uint32_t *__restrict__ modnum, const uint8_t *__restrict__ seqs,
                              uint16_t *__restrict__ code, uint8_t *__restrict__ used)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t c = entry_code(minm, maxm, L, seqs + (size_t)seqid[k] * L, (double)mass[k], modnum[k], sites[k]);
    code[k] = (uint16_t)c;
    used[c] = 1;
}

__global__ void k_entry_classes(const uint16_t *__restrict__ code, uint32_t n, const uint8_t *__restrict__ class_of,
                                uint8_t *__restrict__ cls)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    cls[k] = class_of[code[k]];
}

// the charge of a query posting's ion when it is a y1 ion, else -1;
// ion = series * half + charge * (L - 1) + position
__device__ __forceinline__ int y1_charge(uint32_t ion, uint32_t Lm1, uint32_t half)
{
    if (ion < half || (ion - half) % Lm1) return -1;
    return (int)((ion - half) / Lm1);
}

constexpr uint32_t kPosChunk = 64;  // postings per thread in the flat kernels below

// The bucket holding position i of the query postings, from a bucket b with
// qA[b] <= i: b itself while i is inside it, else the last bucket starting at
// or before i (a binary search, so runs of empty buckets cost no walk).
__device__ __forceinline__ uint32_t bucket_at(const uint32_t *__restrict__ qA, uint32_t nb, uint32_t i, uint32_t b)
{
    if (qA[b + 1] > i) return b;
    uint32_t lo = b + 1, hi = nb;
    while (lo < hi)
    {
        const uint32_t m = (lo + hi + 1) >> 1;
        if (qA[m] <= i) lo = m;
        else hi = m - 1;
    }
    return lo;
}

// kPosChunk postings per thread: every y1 posting of a classed entry must lie
// in its class's key bucket; bad[e] = 1 marks the entries where one does not
// (they lose their class).
__global__ void k_class_check(const uint32_t *__restrict__ qA, const uint32_t *__restrict__ qp,
                              const uint16_t *__restrict__ qion, uint32_t nb, uint32_t total, uint32_t Lm1,
                              uint32_t half, const uint8_t *__restrict__ cls, const ClassKeys *__restrict__ ck,
                              uint8_t *__restrict__ bad)
{
    const uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kPosChunk;
    if (i0 >= total) return;
    const uint32_t i1 = (uint32_t)min((uint64_t)total, i0 + kPosChunk);
    uint32_t b = bucket_at(qA, nb, (uint32_t)i0, 0);
    for (uint32_t i = (uint32_t)i0; i < i1; i++)
    {
        const uint32_t x = qp[i];
        if (x == kQpostPad) continue;
        const int z = y1_charge(qion[i], Lm1, half);
        if (z < 0) continue;
        b = bucket_at(qA, nb, i, b);
        const uint32_t e = x >> kQpEntryShift, c = cls[e];
        if (c != kClassNone && ck->key[c][z] != b) bad[e] = 1;
    }
}

__global__ void k_class_fix(uint8_t *__restrict__ cls, const uint8_t *__restrict__ bad, uint32_t n)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && bad[k]) cls[k] = (uint8_t)kClassNone;
}

// a query posting stays in the search postings unless it is padding or the
// y1 posting of a classed entry
__device__ __forceinline__ bool search_kept(uint32_t x, uint32_t ion, uint32_t Lm1, uint32_t half,
                                            const uint8_t *__restrict__ cls)
{
    if (x == kQpostPad) return false;
    return y1_charge(ion, Lm1, half) < 0 || cls[x >> kQpEntryShift] == kClassNone;
}

// keep[i] = 1 for a query posting that stays in the search postings, else 0
__global__ void k_spost_keep(const uint32_t *__restrict__ qp, const uint16_t *__restrict__ qion, uint32_t total,
                              uint32_t Lm1, uint32_t half, const uint8_t *__restrict__ cls, uint32_t *__restrict__ keep)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        keep[i] = search_kept(qp[i], qion[i], Lm1, half, cls) ? 1u : 0u;
}

// the padded size of each bucket's search postings, from the exclusive scan S
// of the keep flags; entry nb is 0 (the scan makes it the total)
__global__ void k_spost_counts(const uint32_t *__restrict__ qA, const uint32_t *__restrict__ S, uint32_t nb,
                                uint32_t *__restrict__ qAs)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b <= nb; b += gridDim.x * blockDim.x)
        qAs[b] = b < nb ? ((S[qA[b + 1]] - S[qA[b]] + 3u) & ~3u) : 0u;
}

// kPosChunk postings per thread: each kept posting to its place, bucket b's
// at qAs[b] in their order.
__global__ void k_spost_scatter(const uint32_t *__restrict__ qA, const uint32_t *__restrict__ qp,
                                 const uint32_t *__restrict__ S, uint32_t nb, uint32_t total,
                                 const uint32_t *__restrict__ qAs, uint32_t *__restrict__ qps)
{
    const uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kPosChunk;
    if (i0 >= total) return;
    const uint32_t i1 = (uint32_t)min((uint64_t)total, i0 + kPosChunk);
    uint32_t b = bucket_at(qA, nb, (uint32_t)i0, 0);
    for (uint32_t i = (uint32_t)i0; i < i1; i++)
    {
        if (S[i + 1] == S[i]) continue;  // not kept
        b = bucket_at(qA, nb, i, b);
        qps[qAs[b] + S[i] - S[qA[b]]] = qp[i];
    }
}

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    return cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
}

// Device scratch of one build step, freed when the step returns (also on its
// error paths).
struct Scratch
{
    std::vector<void *> ptrs;
    template <class T>
    cudaError_t alloc(T **p, size_t n)
    {
        const cudaError_t e = dalloc(p, n);
        if (e == cudaSuccess) ptrs.push_back(*p);
        else *p = nullptr;
        return e;
    }
    ~Scratch()
    {
        for (void *p : ptrs) cudaFree(p);
    }
};

}  // namespace

// The entries of one length enumerated on the device (k_enum_entries, two
// passes around a scan of the per-peptide variant counts) into fresh SoA
// arrays in generation order; sets lh.n.
static int enumerate_entries(hc_ctx *ctx, LenHost &lh, Scratch &out, float **d_m, uint32_t **d_s,
                             uint64_t **d_si, uint32_t **d_mo, int *launches)
{
    cudaStream_t st = ctx->stream;
    const uint32_t npep = lh.npep, L = lh.L;
    EnumConst ec;
    make_enum_const(ctx->p, &ec);
    Scratch tmp;
    uint32_t *cnt = nullptr, *stmp = nullptr;
    HC_CUDA(ctx, tmp.alloc(&cnt, (size_t)npep + 1));
    HC_CUDA(ctx, tmp.alloc(&stmp, scan_tmp_words((size_t)npep + 1)));
    HC_CUDA(ctx, cudaMemsetAsync(cnt, 0, 4ull * (npep + 1), st));
    const unsigned grid = (npep + 127) / 128;
    if (npep)
    {
        k_enum_entries<<<grid, 128, 0, st>>>(lh.d_seqs, L, npep, ec, nullptr, cnt, nullptr, nullptr, nullptr,
                                              nullptr);
        (*launches)++;
    }
    HC_CUDA(ctx, scan_exclusive(cnt, (size_t)npep + 1, stmp, st));
    uint32_t nvar = 0;
    HC_CUDA(ctx, cudaMemcpyAsync(&nvar, cnt + npep, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    const uint64_t n = (uint64_t)npep + nvar;
    if (n >= (1u << 24)) return set_error(ctx, HC_ERR_INVLD_SIZE, "more than 2^24 entries in one length");
    lh.n = (uint32_t)n;
    HC_CUDA(ctx, out.alloc(d_m, n));
    HC_CUDA(ctx, out.alloc(d_s, n));
    HC_CUDA(ctx, out.alloc(d_si, n));
    HC_CUDA(ctx, out.alloc(d_mo, n));
    if (npep)
    {
        k_enum_entries<<<grid, 128, 0, st>>>(lh.d_seqs, L, npep, ec, cnt, nullptr, *d_m, *d_s, *d_si, *d_mo);
        (*launches)++;
    }
    HC_CUDA(ctx, cudaGetLastError());
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    return HC_SUCCESS;
}

int build_length_device(hc_ctx *ctx, LenHost &lh, const hc_entry *h_entries, bool sort_by_mass)
{
    cudaStream_t st = ctx->stream;
    int launches = 0;
    // entries in generation order: enumerated here, or uploaded from the host
    Scratch scr;
    float *d_m0 = nullptr;
    uint32_t *d_s0 = nullptr, *d_mod0 = nullptr;
    uint64_t *d_site0 = nullptr;
    if (!h_entries)
    {
        const int rc = enumerate_entries(ctx, lh, scr, &d_m0, &d_s0, &d_site0, &d_mod0, &launches);
        if (rc) return rc;
    }
    const uint32_t n = lh.n, L = lh.L;
    const uint32_t speclen = 2 * ctx->p.maxz * (L - 1);
    const size_t M = (size_t)n * speclen;
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    if (M >= 0x80000000ull) return set_error(ctx, HC_ERR_INVLD_SIZE, "more than 2^31 ions in one length");
    if (h_entries && (sort_by_mass && n > 1))
    {
        std::vector<float> hm(n);
        std::vector<uint32_t> hs(n), hmod(n);
        std::vector<uint64_t> hsite(n);
        for (uint32_t i = 0; i < n; i++)
        {
            hm[i] = h_entries[i].mass;
            hs[i] = h_entries[i].seqid;
            hsite[i] = h_entries[i].sites;
            hmod[i] = h_entries[i].modnum;
        }
        HC_CUDA(ctx, scr.alloc(&d_m0, n));
        HC_CUDA(ctx, scr.alloc(&d_s0, n));
        HC_CUDA(ctx, scr.alloc(&d_mod0, n));
        HC_CUDA(ctx, scr.alloc(&d_site0, n));
        HC_CUDA(ctx, cudaMemcpy(d_m0, hm.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(d_s0, hs.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(d_mod0, hmod.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(d_site0, hsite.data(), 8ull * n, cudaMemcpyHostToDevice));
    }
    HC_CUDA(ctx, dalloc(&lh.d_mass, n));
    HC_CUDA(ctx, dalloc(&lh.d_seqid, n));
    HC_CUDA(ctx, dalloc(&lh.d_sites, n));
    HC_CUDA(ctx, dalloc(&lh.d_modnum, n));
    HC_CUDA(ctx, dalloc(&lh.d_bA, (size_t)nb + 1));

    // scratch: keys/vals ping-pong, radix histograms, scan temp
    const size_t items = M > n ? M : n;
    const size_t ntiles = (items + kRsTile - 1) / kRsTile;
    uint32_t *k0, *k1, *v0, *v1, *hist, *stmp, *d_uninit;
    HC_CUDA(ctx, scr.alloc(&k0, items));
    HC_CUDA(ctx, scr.alloc(&k1, items));
    HC_CUDA(ctx, scr.alloc(&v0, items));
    HC_CUDA(ctx, scr.alloc(&v1, items));
    HC_CUDA(ctx, scr.alloc(&hist, ntiles * kRadix));
    HC_CUDA(ctx, scr.alloc(&stmp, scan_tmp_words(ntiles * kRadix)));
    HC_CUDA(ctx, scr.alloc(&d_uninit, 1));
    HC_CUDA(ctx, cudaMemsetAsync(d_uninit, 0, 4, st));

    if (sort_by_mass && n > 1)
    {
        k_mass_keys<<<(n + 255) / 256, 256, 0, st>>>(d_m0, n, k0);
        int which = 0;
        HC_CUDA(ctx, radix_sort(k0, k1, v0, v1, n, 32, hist, stmp, st, &which, &launches, false, true));
        // after an even number of passes the result is in (k0, v0)
        uint32_t *perm = which ? v1 : v0;
        k_gather_entries<<<(n + 255) / 256, 256, 0, st>>>(perm, n, d_m0, d_s0, d_site0, d_mod0,
                                                          lh.d_mass, lh.d_seqid, lh.d_sites,
                                                          lh.d_modnum);
        launches += 2;
    }
    else if (d_m0)
    {
        HC_CUDA(ctx, cudaMemcpyAsync(lh.d_mass, d_m0, 4ull * n, cudaMemcpyDeviceToDevice, st));
        HC_CUDA(ctx, cudaMemcpyAsync(lh.d_seqid, d_s0, 4ull * n, cudaMemcpyDeviceToDevice, st));
        HC_CUDA(ctx, cudaMemcpyAsync(lh.d_modnum, d_mod0, 4ull * n, cudaMemcpyDeviceToDevice, st));
        HC_CUDA(ctx, cudaMemcpyAsync(lh.d_sites, d_site0, 8ull * n, cudaMemcpyDeviceToDevice, st));
    }
    else
    {
        std::vector<float> hm(n);
        std::vector<uint32_t> hs(n), hmod(n);
        std::vector<uint64_t> hsite(n);
        for (uint32_t i = 0; i < n; i++)
        {
            hm[i] = h_entries[i].mass;
            hs[i] = h_entries[i].seqid;
            hsite[i] = h_entries[i].sites;
            hmod[i] = h_entries[i].modnum;
        }
        HC_CUDA(ctx, cudaMemcpy(lh.d_mass, hm.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(lh.d_seqid, hs.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(lh.d_modnum, hmod.data(), 4ull * n, cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(lh.d_sites, hsite.data(), 8ull * n, cudaMemcpyHostToDevice));
    }

    // ion keys -> (k0), sorted with ids -> iA, bucket bounds -> bA
    if (M > 0)
    {
        const uint64_t threads = (uint64_t)n * 2 * ctx->p.maxz;
        k_ion_keys<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(
            ctx->d_tables, L, n, lh.d_mass, lh.d_seqid, lh.d_sites, lh.d_modnum, lh.d_seqs, k0,
            d_uninit);
        launches++;
        int bits = 1;
        while ((1ull << bits) < nb) bits++;
        int which = 0;
        HC_CUDA(ctx, radix_sort(k0, k1, v0, v1, M, bits, hist, stmp, st, &which, &launches, true, true));
        uint32_t *skeys = which ? k1 : k0;
        uint32_t *svals = which ? v1 : v0;
        k_bucket_bounds<<<(unsigned)std::min<uint64_t>((nb + 256) / 256, (uint64_t)ctx->sm_count * 32), 256, 0,
                          st>>>(skeys, M, nb, lh.d_bA);
        launches += 1;
        lh.npost = M;
        const int rq = build_query_postings(ctx, lh, svals);
        if (rq) return rq;
        launches += 4;
    }
    else
    {
        HC_CUDA(ctx, cudaMemsetAsync(lh.d_bA, 0, 4ull * (nb + 1), st));
        lh.npost = 0;
        const int rq = build_query_postings(ctx, lh, nullptr);
        if (rq) return rq;
    }
    uint32_t h_uninit = 0;
    HC_CUDA(ctx, cudaMemcpyAsync(&h_uninit, d_uninit, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    lh.built = true;
    ctx->lens_dirty = true;
    ctx->last_launches = launches + 1;
    return HC_SUCCESS;
}

// The query postings (padded buckets), their bucket starts and the row table,
// from bA (on the device) and the ids in bucket order (d_ids; null when the
// length has no postings). Leaves d_ids untouched.
int build_query_postings(hc_ctx *ctx, LenHost &lh, const uint32_t *d_ids)
{
    cudaStream_t st = ctx->stream;
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    const uint32_t speclen = 2 * ctx->p.maxz * (lh.L - 1);
    // entry << 3 must stay below 2^32 and below the padding word
    if (lh.n > kQpMaxEntries)
        return set_error(ctx, HC_ERR_INVLD_SIZE, "too many entries of one length for the query postings");
    cudaFree(lh.d_qA);
    cudaFree(lh.d_qp);
    cudaFree(lh.d_qion);
    cudaFree(lh.d_rows);
    lh.d_qA = lh.d_qp = lh.d_rows = nullptr;
    lh.d_qion = nullptr;
    HC_CUDA(ctx, dalloc(&lh.d_qA, (size_t)nb + 1));
    uint32_t *stmp = nullptr;
    Scratch scr;
    HC_CUDA(ctx, scr.alloc(&stmp, scan_tmp_words((size_t)nb + 1)));
    const unsigned bblocks = (unsigned)std::min<uint64_t>((nb + 256) / 256, (uint64_t)ctx->sm_count * 16);
    k_pad_counts<<<bblocks, 256, 0, st>>>(lh.d_bA, nb, lh.d_qA);
    HC_CUDA(ctx, scan_exclusive(lh.d_qA, (size_t)nb + 1, stmp, st));
    uint32_t total = 0;
    HC_CUDA(ctx, cudaMemcpyAsync(&total, lh.d_qA + nb, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    HC_CUDA(ctx, dalloc(&lh.d_qp, (size_t)total + kIaPad));
    HC_CUDA(ctx, dalloc(&lh.d_qion, (size_t)total + kIaPad));
    HC_CUDA(ctx, cudaMemsetAsync(lh.d_qp, 0xFF, 4 * ((size_t)total + kIaPad), st));
    HC_CUDA(ctx, cudaMemsetAsync(lh.d_qion, 0, 2 * ((size_t)total + kIaPad), st));
    if (d_ids && lh.npost)
        k_qpost<<<bblocks, 256, 0, st>>>(lh.d_bA, d_ids, lh.d_qA, nb, speclen, speclen / 2, lh.d_qp, lh.d_qion);
    HC_CUDA(ctx, cudaGetLastError());
    return build_rows(ctx, lh);
}

// Classes for the codes seen in `used` that have none yet (ids are only ever
// added, so the lengths built before keep theirs), and the device copies.
static int add_classes(hc_ctx *ctx, const std::vector<uint8_t> &used)
{
    bool changed = false;
    for (uint32_t code = 0; code < kCodes; code++)
    {
        if (!used[code] || code == kCodes - 2 || ctx->class_of[code] != kClassNone || ctx->classes.n >= kMaxClasses)
            continue;
        const uint32_t id = ctx->classes.n++;
        ctx->class_of[code] = (uint8_t)id;
        class_keys_of(ctx->p, ctx->tables, code, ctx->classes.key[id]);
        for (uint32_t z = 0; z < ctx->p.maxz; z++)
            ctx->classes.maxkey = std::max(ctx->classes.maxkey, ctx->classes.key[id][z]);
        changed = true;
    }
    if (!ctx->d_classes)
    {
        HC_CUDA(ctx, cudaMalloc((void **)&ctx->d_classes, sizeof(ClassKeys)));
        HC_CUDA(ctx, cudaMalloc((void **)&ctx->d_class_of, kCodes));
        changed = true;
    }
    if (changed)
    {
        HC_CUDA(ctx, cudaMemcpy(ctx->d_classes, &ctx->classes, sizeof(ClassKeys), cudaMemcpyHostToDevice));
        HC_CUDA(ctx, cudaMemcpy(ctx->d_class_of, ctx->class_of.data(), kCodes, cudaMemcpyHostToDevice));
    }
    return HC_SUCCESS;
}

// The search side of a length from its query postings (qA, qp, qion and the
// entries set): each entry's class (checked against its own y1 postings),
// the search postings (the query postings less the y1 postings of classed
// entries, buckets padded to 4 words) and their row table.
int build_rows(hc_ctx *ctx, LenHost &lh)
{
    cudaStream_t st = ctx->stream;
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale, n = lh.n, Lm1 = lh.L - 1;
    const uint32_t half = ctx->p.maxz * Lm1;
    cudaFree(lh.d_rows);
    cudaFree(lh.d_qAs);
    cudaFree(lh.d_qps);
    cudaFree(lh.d_cls);
    lh.d_rows = lh.d_qAs = lh.d_qps = nullptr;
    lh.d_cls = nullptr;
    HC_CUDA(ctx, dalloc(&lh.d_cls, (size_t)n + 4));  // +4: the search reads class bytes in fours
    HC_CUDA(ctx, dalloc(&lh.d_qAs, (size_t)nb + 1));
    HC_CUDA(ctx, cudaMemsetAsync(lh.d_cls, (int)kClassNone, (size_t)n + 4, st));
    const unsigned eblocks = (n + 255) / 256;
    uint32_t qtotal = 0;  // query postings with padding
    HC_CUDA(ctx, cudaMemcpyAsync(&qtotal, lh.d_qA + nb, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    const unsigned pblocks = (unsigned)(((uint64_t)qtotal + 256ull * kPosChunk - 1) / (256ull * kPosChunk));
    Scratch scr;
    if (n > 0)
    {
        uint16_t *code;
        uint8_t *used, *bad;
        HC_CUDA(ctx, scr.alloc(&code, n));
        HC_CUDA(ctx, scr.alloc(&used, (size_t)kCodes));
        HC_CUDA(ctx, scr.alloc(&bad, (size_t)n));
        HC_CUDA(ctx, cudaMemsetAsync(used, 0, kCodes, st));
        HC_CUDA(ctx, cudaMemsetAsync(bad, 0, n, st));
        k_entry_codes<<<eblocks, 256, 0, st>>>((double)ctx->p.min_mass, (double)ctx->p.max_mass, lh.L, n, lh.d_mass,
                                              lh.d_seqid, lh.d_sites, lh.d_modnum, lh.d_seqs, code, used);
        HC_CUDA(ctx, cudaGetLastError());
        std::vector<uint8_t> hused(kCodes);
        HC_CUDA(ctx, cudaMemcpyAsync(hused.data(), used, kCodes, cudaMemcpyDeviceToHost, st));
        HC_CUDA(ctx, cudaStreamSynchronize(st));
        const int rc = add_classes(ctx, hused);
        if (rc) return rc;
        k_entry_classes<<<eblocks, 256, 0, st>>>(code, n, ctx->d_class_of, lh.d_cls);
        if (qtotal)
            k_class_check<<<pblocks, 256, 0, st>>>(lh.d_qA, lh.d_qp, lh.d_qion, nb, qtotal, Lm1, half, lh.d_cls,
                                                   ctx->d_classes, bad);
        k_class_fix<<<eblocks, 256, 0, st>>>(lh.d_cls, bad, n);
        HC_CUDA(ctx, cudaGetLastError());
    }
    // keep flags of the query postings, their exclusive scan S (S[qtotal] =
    // postings kept), the padded bucket sizes from S and their scan (qAs),
    // then every kept posting to its place
    uint32_t *keep = nullptr, *stmp = nullptr, *btmp = nullptr;
    HC_CUDA(ctx, scr.alloc(&keep, (size_t)qtotal + 1));
    HC_CUDA(ctx, scr.alloc(&stmp, scan_tmp_words((size_t)qtotal + 1)));
    HC_CUDA(ctx, scr.alloc(&btmp, scan_tmp_words((size_t)nb + 1)));
    HC_CUDA(ctx, cudaMemsetAsync(keep + qtotal, 0, 4, st));
    if (qtotal)
        k_spost_keep<<<(unsigned)std::min<uint64_t>((qtotal + 255) / 256, (uint64_t)ctx->sm_count * 64), 256, 0, st>>>(
            lh.d_qp, lh.d_qion, qtotal, Lm1, half, lh.d_cls, keep);
    HC_CUDA(ctx, cudaGetLastError());
    HC_CUDA(ctx, scan_exclusive(keep, (size_t)qtotal + 1, stmp, st));
    k_spost_counts<<<(unsigned)std::min<uint64_t>((nb + 256) / 256, (uint64_t)ctx->sm_count * 16), 256, 0, st>>>(
        lh.d_qA, keep, nb, lh.d_qAs);
    HC_CUDA(ctx, cudaGetLastError());
    HC_CUDA(ctx, scan_exclusive(lh.d_qAs, (size_t)nb + 1, btmp, st));
    uint32_t total = 0;
    HC_CUDA(ctx, cudaMemcpyAsync(&total, lh.d_qAs + nb, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    lh.nsearch = total;
    HC_CUDA(ctx, dalloc(&lh.d_qps, (size_t)total + kIaPad));
    HC_CUDA(ctx, cudaMemsetAsync(lh.d_qps, 0xFF, 4 * ((size_t)total + kIaPad), st));
    if (qtotal)
        k_spost_scatter<<<pblocks, 256, 0, st>>>(lh.d_qA, lh.d_qp, keep, nb, qtotal, lh.d_qAs, lh.d_qps);
    HC_CUDA(ctx, cudaGetLastError());
    lh.stride = (n + kRowG - 1) / kRowG + 1;
    HC_CUDA(ctx, dalloc(&lh.d_rows, (size_t)nb * lh.stride));
    const uint64_t rt = (uint64_t)nb * lh.stride;
    const unsigned blocks = (unsigned)std::min<uint64_t>((rt + 255) / 256, (uint64_t)ctx->sm_count * 64);
    k_row_table<<<blocks, 256, 0, st>>>(lh.d_qAs, lh.d_qps, nb, lh.stride, n, lh.d_rows);
    HC_CUDA(ctx, cudaGetLastError());
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    return HC_SUCCESS;
}

// Checks query postings read from outside (an index file): bucket starts
// ascending multiples of 4 ending at the total, and every word padding or a
// valid (entry, ion). Returns HC_ERR_FILE_ERROR otherwise.
int check_query_postings(hc_ctx *ctx, const LenHost &lh, uint64_t qtotal)
{
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    const uint32_t speclen = 2 * ctx->p.maxz * (lh.L - 1);
    if (lh.n > kQpMaxEntries)
        return set_error(ctx, HC_ERR_FILE_ERROR, "index file: too many entries of one length");
    std::vector<uint32_t> qa(nb + 1);
    HC_CUDA(ctx, cudaMemcpy(qa.data(), lh.d_qA, 4ull * (nb + 1), cudaMemcpyDeviceToHost));
    for (uint32_t b = 0; b <= nb; b++)
        if ((qa[b] & 3u) || (b && qa[b] < qa[b - 1]))
            return set_error(ctx, HC_ERR_FILE_ERROR, "index file: bucket starts out of order");
    if (qa[0] != 0 || qa[nb] != qtotal) return set_error(ctx, HC_ERR_FILE_ERROR, "index file: bucket starts");
    uint32_t *d_bad = nullptr;
    HC_CUDA(ctx, cudaMalloc((void **)&d_bad, 4));
    uint32_t bad = 0;
    cudaError_t e = cudaMemset(d_bad, 0, 4);
    if (e == cudaSuccess && qtotal)
    {
        const unsigned blocks = (unsigned)std::min<uint64_t>((qtotal + 255) / 256, (uint64_t)ctx->sm_count * 32);
        k_check_qpost<<<blocks, 256, 0, ctx->stream>>>(lh.d_qp, lh.d_qion, qtotal, lh.n, speclen, speclen / 2, d_bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    HC_CUDA(ctx, e);
    if (bad) return set_error(ctx, HC_ERR_FILE_ERROR, "index file: invalid postings");
    return HC_SUCCESS;
}

// The reference's iA (ids entry*speclen + ion, bucket order) from the query postings.
int export_ids(hc_ctx *ctx, const LenHost &lh, uint32_t *d_ids)
{
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    const uint32_t speclen = 2 * ctx->p.maxz * (lh.L - 1);
    const unsigned bblocks = (unsigned)std::min<uint64_t>((nb + 255) / 256, (uint64_t)ctx->sm_count * 16);
    if (lh.npost)
        k_qpost_ids<<<bblocks, 256, 0, ctx->stream>>>(lh.d_bA, lh.d_qA, lh.d_qp, lh.d_qion, nb, speclen, d_ids);
    HC_CUDA(ctx, cudaGetLastError());
    HC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HC_SUCCESS;
}

}  // namespace hc
