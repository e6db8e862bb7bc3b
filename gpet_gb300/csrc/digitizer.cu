// digitizer.cu - the digitizer chain and the coincidence sorter on the device
// (the work gPET.cu:385-424 does with blur/energywindow/setSitenum/deadtime
// kernels and four host std::sort round trips), for sm_103a.
//
//   blur + threshold      one pass, draws keyed by (parn, slot)
//   time order            stable LSD radix sort on the IEEE bits of t
//                         (8 passes of 8 bits), equal-t runs ordered by
//                         (parn, slot): total order (t, parn, slot)
//   site order            stable radix sort of the time order by site
//   dead time             paralyzable: one comparison with the previous
//                         pulse of the site; non-paralyzable: one thread per
//                         cluster (a pulse >= tau after its predecessor starts
//                         a cluster no earlier pulse can reach)
//   energy window         ordered compaction of the time order
//   coincidences          one thread per cluster of singles closer than the
//                         window; pair counts, scan, write
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "../../include/gpet.h"

namespace gpet {

constexpr int kTile = 4096;      // items per block in radix / scan kernels
// time keys: (t - tmin) quantised to 32 bits over the survivors' time span
// (4 radix passes instead of 8 on the IEEE bits); runs of equal keys are
// ordered by (t, parn, slot) after the sort. m pulses spread over the span
// share a key with m / 2^32 others on average (about 1e-3 for a 1e8-decay
// acquisition), so the runs are the few pulses of one instant.
constexpr int kTimeKeyBits = 32;
constexpr uint64_t kTimeKeyMax = (1ull << kTimeKeyBits) - 1;

static unsigned grid_for(int64_t n, int threads);
constexpr int kScanThreads = 1024;

// ---------------------------------------------------------------- scan
__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ aux)
{
    __shared__ uint32_t ws[32];
    int64_t base = (int64_t)blockIdx.x * kTile;
    uint32_t s = 0;
    for (int k = threadIdx.x; k < kTile; k += blockDim.x) {
        int64_t i = base + k;
        if (i < n) s += in[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) aux[blockIdx.x] = v;
    }
}

// block-wide exclusive scan of one value per thread (blockDim.x == 1024)
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t* ws, uint32_t& total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t x = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
        uint32_t xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += t;
        }
        ws[lane] = xi - x;
        if (lane == 31) ws[32] = xi;
    }
    __syncthreads();
    uint32_t r = ws[w] + inc - v;
    total = ws[32];
    __syncthreads();
    return r;
}

// exclusive scan of the per-block sums, single block
__global__ void k_scan_aux(uint32_t* aux, int64_t nb, uint32_t* total)
{
    __shared__ uint32_t ws[33];
    uint32_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        int64_t i = b0 + threadIdx.x;
        uint32_t v = i < nb ? aux[i] : 0;
        uint32_t tot;
        uint32_t e = block_exscan(v, ws, tot);
        if (i < nb) aux[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_down(const uint32_t* in, int64_t n, const uint32_t* __restrict__ aux, uint32_t* out)
{
    __shared__ uint32_t ws[33];
    int64_t base = (int64_t)blockIdx.x * kTile;
    uint32_t carry = aux[blockIdx.x];
    constexpr int per = kTile / kScanThreads;   // 4 consecutive items per thread
    uint32_t v[per];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < per; ++k) {
        int64_t i = base + (int64_t)threadIdx.x * per + k;
        v[k] = i < n ? in[i] : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t e = block_exscan(s, ws, tot);
    uint32_t run = carry + e;
#pragma unroll
    for (int k = 0; k < per; ++k) {
        int64_t i = base + (int64_t)threadIdx.x * per + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

// exclusive scan in -> out (may alias), total written to *total (device)
static void scan_exclusive(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* aux, uint32_t* total,
                           cudaStream_t s, int64_t* launches)
{
    int64_t nb = (n + kTile - 1) / kTile;
    if (nb == 0) {
        cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return;
    }
    k_scan_reduce<<<(unsigned)nb, 256, 0, s>>>(in, n, aux);
    k_scan_aux<<<1, kScanThreads, 0, s>>>(aux, nb, total);
    k_scan_down<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, aux, out);
    *launches += 3;
}

// ---------------------------------------------------------------- radix sort
__global__ void __launch_bounds__(256) k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                                    uint32_t* __restrict__ hist, int64_t nblocks)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kTile;
    for (int k = threadIdx.x; k < kTile; k += 256) {
        int64_t i = base + k;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// stable scatter: items of a tile keep their order within a digit. The tile
// is first reordered by digit in shared memory, then written out in that
// order, so the threads of a warp write consecutive addresses of a digit's
// run instead of 32 scattered ones.
constexpr int kScatterSmem = kTile * (8 + 4);   // the tile's keys and values

__global__ void __launch_bounds__(256) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                       const uint32_t* __restrict__ vin, int64_t n, int shift,
                                                       const uint32_t* __restrict__ off, int64_t nblocks,
                                                       uint64_t* __restrict__ kout, uint32_t* __restrict__ vout)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    uint64_t* sk = reinterpret_cast<uint64_t*>(dsm);
    uint32_t* sv = reinterpret_cast<uint32_t*>(dsm + kTile * 8);
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[8][256];
    __shared__ uint32_t soff[256];   // where this tile's run of digit d starts in the output
    __shared__ uint32_t toff[256];   // where it starts within the tile
    __shared__ uint32_t wsum[8];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const int64_t base = (int64_t)blockIdx.x * kTile;
    const int ntile = (int)(n - base < kTile ? n - base : kTile);
    // the tile's count of digit tid: the scanned histogram is digit-major, so
    // its next entry is this one plus that count (n after the last)
    const int64_t fi = (int64_t)tid * nblocks + blockIdx.x;
    const uint32_t g0 = off[fi];
    const uint32_t cnt = (fi + 1 < 256 * nblocks ? off[fi + 1] : (uint32_t)n) - g0;
    soff[tid] = g0;
    run[tid] = 0;
    uint32_t v = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    uint32_t add0 = 0;
    for (int ww = 0; ww < w; ++ww) add0 += wsum[ww];
    toff[tid] = v - cnt + add0;
    for (int r = 0; r < kTile / 256; ++r) {
#pragma unroll
        for (int ww = 0; ww < 8; ++ww) wc[ww][tid] = 0;
        __syncthreads();
        const int li = r * 256 + tid;
        const bool valid = li < ntile;
        const uint64_t key = valid ? kin[base + li] : 0ull;
        const uint32_t val = valid ? vin[base + li] : 0u;
        const uint32_t dig = valid ? (uint32_t)((key >> shift) & 255u) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dig);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) wc[w][dig] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pre = run[dig] + rank;
            for (int ww = 0; ww < w; ++ww) pre += wc[ww][dig];
            const uint32_t lp = toff[dig] + pre;
            sk[lp] = key;
            sv[lp] = val;
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int ww = 0; ww < 8; ++ww) add += wc[ww][tid];
        run[tid] += add;
    }
    __syncthreads();
    for (int li = tid; li < ntile; li += 256) {
        const uint64_t key = sk[li];
        const uint32_t dig = (uint32_t)((key >> shift) & 255u);
        const uint32_t pos = soff[dig] + ((uint32_t)li - toff[dig]);
        kout[pos] = key;
        vout[pos] = sv[li];
    }
}

// sort (keys, vals) of length n by bits [0, nbits) of key, stably; result in
// (ka, va) on return (the buffers are ping-ponged)
void radix_sort(uint64_t*& ka, uint32_t*& va, uint64_t*& kb, uint32_t*& vb, int64_t n, int nbits, uint32_t* hist,
                uint32_t* aux, uint32_t* total, cudaStream_t s, int64_t* launches)
{
    if (n <= 1) return;
    cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, kScatterSmem);
    int64_t nb = (n + kTile - 1) / kTile;
    for (int shift = 0; shift < nbits; shift += 8) {
        k_radix_hist<<<(unsigned)nb, 256, 0, s>>>(ka, n, shift, hist, nb);
        scan_exclusive(hist, hist, 256 * nb, aux, total, s, launches);
        k_radix_scatter<<<(unsigned)nb, 256, kScatterSmem, s>>>(ka, va, n, shift, hist, nb, kb, vb);
        *launches += 2;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
}

// order-preserving unsigned image of a double (negative values included)
__device__ __forceinline__ unsigned long long ordered_bits(double t)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(t);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

static double from_ordered_bits(unsigned long long o)
{
    const unsigned long long u = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    double t;
    std::memcpy(&t, &u, 8);
    return t;
}

// ---------------------------------------------------------------- stages
__device__ __forceinline__ int pulse_sim(const PulseDev& P, int64_t i) { return P.sim ? P.sim[i] : 0; }

// blur (gPET_kernals.cu:814-837) + threshold (energywindow :641-656 with
// [Eth, 2 MeV]); survivors' pulse indices appended to sel, site stored.
// Parameters per simulation: prms[sim].
// range[0], range[1]: smallest and largest ordered_bits of the survivors'
// times, range[2]: their largest site (as unsigned); one atomic per block each
__global__ void k_blur_threshold(PulseDev P, int64_t n, const DigiParams* __restrict__ prms, float* Eb, float* xb,
                                 float* yb, float* zb, int32_t* site, uint32_t* sel, unsigned long long* nsel,
                                 unsigned long long* range)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    // survivors are appended with one atomic per block and iteration (one
    // per warp, all on one counter, made the kernel wait on the atomics)
    __shared__ unsigned s_woff[32];
    __shared__ unsigned long long s_base;
    unsigned long long tlo = ~0ull, thi = 0ull, smax = 0ull;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool keep = false;
        if (i < n) {
            const DigiParams& prm = prms[pulse_sim(P, i)];
            const int32_t parn = P.parn[i];
            const uint32_t slot = P.meta[i] & 0x7fu;
            float E = P.E[i], x = P.x[i], y = P.y[i], z = P.z[i];
            if (parn >= 0) {   // background singles (parn -1) carry their own energy spread
                Stream st;
                st_init(st, prm.key0, prm.key1, kTagBlur, ((uint64_t)(uint32_t)parn << 4) | slot);
                float R = 0.0f;
                if (prm.blurpolicy == 0) R = dm_sqrt(prm.Eref / E) * prm.Rref;
                if (prm.blurpolicy == 1) R = prm.Rref + prm.Eslope * (E - prm.Eref) / 1.0e6f;
                if (R < 0.0f) R = 0.0f;
                float zn = st_normal(st);
                E += zn * R * E / 2.35482f;
                if (prm.Sblur > 0.0f) {
                    x += prm.Sblur * st_normal(st);
                    y += prm.Sblur * st_normal(st);
                    z += prm.Sblur * st_normal(st);
                }
            }
            Eb[i] = E; xb[i] = x; yb[i] = y; zb[i] = z;
            keep = !(E < prm.Eth || E > 2000000.0f);
            // setSitenum, gPET_kernals.cu:607-640 (level 3 keeps the readout site)
            int32_t sv;
            switch (prm.dlevel) {
            case 0: sv = 0; break;
            case 1: sv = P.pann[i]; break;
            case 2: sv = P.pann[i] * prm.moduleN + P.modn[i]; break;
            default: sv = P.siten[i]; break;
            }
            site[i] = sv;
            if (keep) {
                const unsigned long long o = ordered_bits(P.t[i]);
                tlo = o < tlo ? o : tlo;
                thi = o > thi ? o : thi;
                smax = (unsigned long long)(uint32_t)sv > smax ? (unsigned long long)(uint32_t)sv : smax;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) s_woff[wid] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (int k = 0; k < nwarps; ++k) {
                const unsigned c = s_woff[k];
                s_woff[k] = tot;
                tot += c;
            }
            s_base = tot ? atomicAdd(nsel, (unsigned long long)tot) : 0ull;
        }
        __syncthreads();
        if (keep) sel[s_base + s_woff[wid] + __popc(m & lt)] = (uint32_t)i;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, tlo, o);
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, thi, o);
        const unsigned long long z = __shfl_xor_sync(0xffffffffu, smax, o);
        tlo = x < tlo ? x : tlo;
        thi = y > thi ? y : thi;
        smax = z > smax ? z : smax;
    }
    __shared__ unsigned long long red[3][32];
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        red[0][w] = tlo;
        red[1][w] = thi;
        red[2][w] = smax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; ++k) {
            tlo = red[0][k] < tlo ? red[0][k] : tlo;
            thi = red[1][k] > thi ? red[1][k] : thi;
            smax = red[2][k] > smax ? red[2][k] : smax;
        }
        if (thi) {
            atomicMin(&range[0], tlo);
            atomicMax(&range[1], thi);
            atomicMax(&range[2], smax);
        }
    }
}

// time keys: with quant, floor((t - tmin) * scale) (at most 32 bits; t >=
// tmin for every selected pulse, and the key is monotone in t), else the
// IEEE bits of t (non-negative times order like their bits)
__global__ void k_time_keys(const uint32_t* __restrict__ sel, int64_t m, const double* __restrict__ t, int quant,
                            double tmin, double scale, uint64_t* key, uint32_t* val)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = sel[j];
        if (quant) {
            const double x = (t[p] - tmin) * scale;
            uint64_t q = x > 0.0 ? (uint64_t)x : 0ull;
            key[j] = q > kTimeKeyMax ? kTimeKeyMax : q;
        } else {
            key[j] = (uint64_t)__double_as_longlong(t[p]);
        }
        val[j] = p;
    }
}

// order each run of equal keys by (t, parn, slot) (quantised keys can join
// different times; equal IEEE keys are equal times)
__global__ void k_tie_fix(const uint64_t* __restrict__ key, uint32_t* idx, int64_t m, const double* __restrict__ t,
                          const int32_t* __restrict__ parn, const uint8_t* __restrict__ meta)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        if (j > 0 && key[j] == key[j - 1]) continue;
        if (j + 1 >= m || key[j + 1] != key[j]) continue;
        int64_t e = j + 1;
        while (e < m && key[e] == key[j]) e++;
        for (int64_t a = j + 1; a < e; ++a) {
            const uint32_t v = idx[a];
            const double tv = t[v];
            const uint64_t kv = ((uint64_t)(uint32_t)parn[v] << 8) | (meta[v] & 0x7fu);
            int64_t b = a - 1;
            while (b >= j) {
                const uint32_t u = idx[b];
                const double tu = t[u];
                const uint64_t ku = ((uint64_t)(uint32_t)parn[u] << 8) | (meta[u] & 0x7fu);
                if (tu < tv || (tu == tv && ku <= kv)) break;
                idx[b + 1] = u;
                b--;
            }
            idx[b + 1] = v;
        }
    }
}

// keys of the time order of the m selected pulses from the survivors' time
// range (host copy of k_blur_threshold's range[0..1]); returns the key bits
int launch_time_keys(const uint32_t* sel, int64_t m, const double* t, const unsigned long long* range,
                     uint64_t* key, uint32_t* val, cudaStream_t s)
{
    const double tmin = from_ordered_bits(range[0]), tmax = from_ordered_bits(range[1]);
    const double span = tmax - tmin;
    const double scale = (double)kTimeKeyMax / span;
    const bool quant = m > 1 && span > 0.0 && std::isfinite(span) && std::isfinite(scale);
    k_time_keys<<<grid_for(m, 256), 256, 0, s>>>(sel, m, t, quant ? 1 : 0, tmin, quant ? scale : 0.0, key, val);
    return quant ? kTimeKeyBits : 64;
}

// bits of the site keys for sites up to smax
int site_key_bits(unsigned long long smax)
{
    int bits = 8;
    while (bits < 32 && (1ull << bits) <= smax) bits += 8;
    return bits;
}

// keys for the stable sort of the time order by simulation
__global__ void k_sim_keys(const uint32_t* __restrict__ order, int64_t m, const int32_t* __restrict__ psim,
                           uint64_t* key, uint32_t* val)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t p = order[j];
        key[j] = (uint64_t)(uint32_t)psim[p];
        val[j] = p;
    }
}

// (simulation, site) keys for the dead-time order
__global__ void k_site_keys(const uint32_t* __restrict__ torder, int64_t m, const int32_t* __restrict__ site,
                            const int32_t* __restrict__ psim, uint64_t* key, uint32_t* val)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t p = torder[j];
        uint64_t sm = psim ? (uint64_t)(uint32_t)psim[p] : 0ull;
        key[j] = (sm << 32) | (uint64_t)(uint32_t)site[p];
        val[j] = p;
    }
}

// per-simulation count of the elements of an order sorted by simulation
__global__ void k_count_by_sim(const uint32_t* __restrict__ order, int64_t m, const int32_t* __restrict__ psim,
                               Counters* cnt, int field)
{
    SimTally t;   // per thread, flushed once
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        t.add(cnt, field, psim ? psim[order[j]] : 0, 1u);
    t.flush(cnt, field);
}

__global__ void k_add_count(Counters* cnt, int field, unsigned long long v)
{
    reinterpret_cast<unsigned long long*>(cnt)[field] += v;
}

// dead time (deadtime, gPET_kernals.cu:657-698, sequential semantics, FP64):
// sorder is the (simulation, site, t, parn, slot) order
// skey: the sorted (simulation, site) keys beside sorder (equal keys: the
// same site of the same simulation); multi: the key's high word is the
// simulation. A pulse's predecessor in this order comes from the lane below
// (key and time), so a pulse costs one gather of its time.
__global__ void k_deadtime(const uint32_t* __restrict__ sorder, const uint64_t* __restrict__ skey, int64_t m,
                           const double* __restrict__ t, const DigiParams* __restrict__ prms, int multi,
                           uint32_t* flags, Counters* cnt)
{
    const int lane = threadIdx.x & 31;
    SimTally t_alive;   // per thread, flushed once (an atomic per warp and iteration queued on one counter)
    // all lanes of a warp run the same iterations (base is block-uniform)
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = base + threadIdx.x;
        const bool in = j < m;
        const uint32_t p = in ? sorder[j] : 0u;
        const uint64_t kp = in ? skey[j] : 0ull;
        const double tp = in ? t[p] : 0.0;
        uint64_t kq = __shfl_up_sync(0xffffffffu, kp, 1);
        double tq = __shfl_up_sync(0xffffffffu, tp, 1);
        if (lane == 0 && in && j > 0) {
            kq = skey[j - 1];
            tq = t[sorder[j - 1]];
        }
        if (!in) continue;
        unsigned alive = 0;
        const int sim = multi ? (int)(kp >> 32) : 0;
        const double tau = prms[sim].tau;
        if (prms[sim].dtype == 0) {
            const bool keep = !(j > 0 && kq == kp && tp < tq + tau);
            flags[p] = keep ? 1u : 0u;
            alive += keep;
        } else {
            // anchors: first pulse of a site or >= tau after its predecessor
            const bool anchor = j == 0 || kq != kp || !(tp < tq + tau);
            if (anchor) {
                double tdead = tp, tprev = tp;
                flags[p] = 1u;
                alive++;
                for (int64_t i = j + 1; i < m; ++i) {
                    const uint32_t a = sorder[i];
                    const double ta = t[a];
                    if (skey[i] != kp || !(ta < tprev + tau)) break;   // next anchor
                    if (ta < tdead + tau) {
                        flags[a] = 0u;
                    } else {
                        flags[a] = 1u;
                        alive++;
                        tdead = ta;
                    }
                    tprev = ta;
                }
            }
        }
        t_alive.add(cnt, CF(n_dead), sim, alive);
    }
    t_alive.flush(cnt, CF(n_dead));
}

// energy window (gPET.cu:418) predicate over the (simulation, t) order
__global__ void k_window_pred(const uint32_t* __restrict__ torder, int64_t m, const uint32_t* __restrict__ flags,
                              const float* __restrict__ Eb, const int32_t* __restrict__ psim,
                              const DigiParams* __restrict__ prms, uint32_t* pred, Counters* cnt)
{
    SimTally t_single;   // per thread, flushed once
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < m; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = base + threadIdx.x;
        if (j < m) {
            const uint32_t p = torder[j];
            const int sim = psim ? psim[p] : 0;
            const float E = Eb[p];
            const bool ok = flags[p] && !(E < prms[sim].ewin_lo || E > prms[sim].ewin_hi);
            pred[j] = ok ? 1u : 0u;
            t_single.add(cnt, CF(n_single), sim, ok ? 1u : 0u);
        }
    }
    t_single.flush(cnt, CF(n_single));
}

__global__ void k_compact(const uint32_t* __restrict__ torder, const uint32_t* __restrict__ pred,
                          const uint32_t* __restrict__ off, int64_t m, uint32_t* out)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
        if (pred[j]) out[off[j]] = torder[j];
}

// coincidence windows (no counterpart in the reference): a single not inside
// an open window opens [t, t+W). One thread walks each cluster of singles
// (a single >= W after its predecessor, or the first of its simulation,
// cannot be inside an earlier window).
__global__ void k_coinc_count(const uint32_t* __restrict__ sidx, int64_t s, const double* __restrict__ t,
                              const int32_t* __restrict__ pann, const int32_t* __restrict__ psim,
                              const DigiParams* __restrict__ prms, uint32_t* wcount, uint32_t* wend, Counters* cnt)
{
    SimTally mult;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < s; j += (int64_t)gridDim.x * blockDim.x) {
        const int sim = psim ? psim[sidx[j]] : 0;
        const double W = prms[sim].window;
        const int policy = prms[sim].coinc_policy;
        auto same_sim = [&](int64_t a, int64_t b) { return !psim || psim[sidx[a]] == psim[sidx[b]]; };
        bool anchor = j == 0 || !same_sim(j, j - 1) || !(t[sidx[j]] < t[sidx[j - 1]] + W);
        if (!anchor) continue;
        int64_t i = j;
        while (i < s && (i == j || (same_sim(i, i - 1) && t[sidx[i]] < t[sidx[i - 1]] + W))) {
            const double ti = t[sidx[i]];
            int64_t e = i + 1;
            while (e < s && same_sim(e, i) && t[sidx[e]] < ti + W) e++;
            const int64_t cnt_w = e - i;
            uint32_t pairs = 0;
            if (policy == 0) {
                if (cnt_w == 2 && pann[sidx[i]] != pann[sidx[i + 1]]) pairs = 1;
            } else {
                for (int64_t a = i; a < e; ++a)
                    for (int64_t b = a + 1; b < e; ++b) pairs += pann[sidx[a]] != pann[sidx[b]];
            }
            mult.add(cnt, CF(n_mult), sim, cnt_w > 2 ? 1u : 0u);
            wcount[i] = pairs;
            wend[i] = (uint32_t)e;
            i = e;
        }
    }
    mult.flush(cnt, CF(n_mult));
}

__global__ void k_coinc_write(const uint32_t* __restrict__ sidx, int64_t s, const uint32_t* __restrict__ wend,
                              const uint32_t* __restrict__ off, const int32_t* __restrict__ pann,
                              const int32_t* __restrict__ eid, const uint8_t* __restrict__ meta,
                              const int32_t* __restrict__ psim, const DigiParams* __restrict__ prms,
                              int64_t* pairs, uint8_t* klass, int64_t cap, Counters* cnt)
{
    SimTally c0, c1, c2;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < s; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = wend[j];
        if (e <= j) continue;
        const int sim = psim ? psim[sidx[j]] : 0;
        const int64_t cnt_w = e - j;
        if (prms[sim].coinc_policy == 0 && cnt_w != 2) continue;
        uint32_t o = off[j];
        for (int64_t a = j; a < e; ++a) {
            for (int64_t b = a + 1; b < e; ++b) {
                const uint32_t pa = sidx[a], pb = sidx[b];
                if (pann[pa] == pann[pb]) continue;
                uint8_t k;
                if (eid[pa] == eid[pb] && eid[pa] >= 0) k = ((meta[pa] | meta[pb]) & 0x80u) ? 1 : 0;
                else k = 2;
                if (o < cap) {
                    pairs[2 * (int64_t)o] = a;
                    pairs[2 * (int64_t)o + 1] = b;
                    klass[o] = k;
                }
                o++;
                c0.add(cnt, CF(n_true), sim, k == 0);
                c1.add(cnt, CF(n_scat), sim, k == 1);
                c2.add(cnt, CF(n_rand), sim, k == 2);
            }
        }
    }
    c0.flush(cnt, CF(n_true));
    c1.flush(cnt, CF(n_scat));
    c2.flush(cnt, CF(n_rand));
}

// ---------------------------------------------------------------- background singles
// events of interval i; with P, written from index o on
__device__ int noise_interval(const NoiseParams& np, int64_t i, const PulseDev* P, int64_t o)
{
    Stream st;
    st_init(st, np.key0, np.key1, kTagNoise, (uint64_t)i);
    double t = np.t0_us + (double)i * np.interval_us;
    double te = np.t0_us + (double)(i + 1) * np.interval_us;
    if (te > np.t1_us) te = np.t1_us;
    int k = 0;
    for (; k < kMaxNoisePerInterval; ++k) {
        const float u = st_u(st);
        t += (double)(-np.lambda_us * dm_logf(u));
        if (!(t < te)) break;
        if (!P) {   // count only: skip the event's eight draws
            for (int d = 0; d < 8; ++d) (void)st_next(st);
            continue;
        }
        const float E = np.emean + np.sigma * st_normal(st);
        const float x = st_u(st);
        const float y = st_u(st);
        const float z = st_u(st);
        int pann = (int)((float)np.npanels * st_u(st));
        int modn = (int)((float)np.moduleN * st_u(st));
        int cryn = (int)((float)np.crystalN * st_u(st));
        pann = pann > np.npanels - 1 ? np.npanels - 1 : pann;
        modn = modn > np.moduleN - 1 ? np.moduleN - 1 : modn;
        cryn = cryn > np.crystalN - 1 ? np.crystalN - 1 : cryn;
        const int64_t j = o + k;
        P->parn[j] = -1;
        P->pann[j] = pann;
        P->modn[j] = modn;
        P->cryn[j] = cryn;
        P->siten[j] = pann * np.moduleN * np.crystalN + modn * np.crystalN + cryn;
        P->eventid[j] = -1;
        P->t[j] = t;
        P->E[j] = E;
        P->x[j] = x;
        P->y[j] = y;
        P->z[j] = z;
        P->meta[j] = 0;
        if (P->sim) P->sim[j] = np.sim;
    }
    return k;
}

__global__ void k_noise_count(NoiseParams np, uint32_t* cnt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np.nint; i += (int64_t)gridDim.x * blockDim.x)
        cnt[i] = (uint32_t)noise_interval(np, i, nullptr, 0);
}

__global__ void k_noise_write(NoiseParams np, const uint32_t* __restrict__ off, PulseDev P, int64_t base, Counters* cnt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np.nint; i += (int64_t)gridDim.x * blockDim.x) {
        const int k = noise_interval(np, i, &P, base + off[i]);
        if (k) atomicAdd(&cnt[np.sim].n_noise, (unsigned long long)k);
    }
}

static unsigned grid_for_g(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

// gather records (gPET.h:87-92 layout) for the pulses listed in idx (or
// 0..n-1); blurred fields and the dead-time site when `blurred`
__global__ void k_gather_events(PulseDev P, const uint32_t* __restrict__ idx, int64_t n, int blurred,
                                const float* __restrict__ Eb, const float* __restrict__ xb,
                                const float* __restrict__ yb, const float* __restrict__ zb,
                                const int32_t* __restrict__ site, EventRec* out, uint8_t* meta)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = idx ? (int64_t)idx[j] : j;
        EventRec e;
        e.parn = P.parn[p]; e.pann = P.pann[p]; e.modn = P.modn[p]; e.cryn = P.cryn[p];
        e.siten = blurred ? site[p] : P.siten[p];
        e.eventid = P.eventid[p];
        e.t = P.t[p];
        if (blurred) { e.E = Eb[p]; e.x = xb[p]; e.y = yb[p]; e.z = zb[p]; }
        else { e.E = P.E[p]; e.x = P.x[p]; e.y = P.y[p]; e.z = P.z[p]; }
        out[j] = e;
        meta[j] = P.meta[p];
    }
}

// the same records for a destination in mapped (pinned) host memory or a
// device buffer: a block builds 256 records in shared memory and stores them
// as consecutive 16-byte words, so every store (across the host link, or to
// device memory) is a whole, aligned word and a warp's stores are coalesced;
// flags[j] = 1 for a record whose photon scattered in the phantom (meta bit 7).
// out must be 16-byte aligned.
__global__ void __launch_bounds__(256) k_gather_events_mapped(PulseDev P, const uint32_t* __restrict__ idx, int64_t n,
                                                              const float* __restrict__ Eb,
                                                              const float* __restrict__ xb,
                                                              const float* __restrict__ yb,
                                                              const float* __restrict__ zb,
                                                              const int32_t* __restrict__ site, uint4* out,
                                                              uint8_t* flags)
{
    __shared__ EventRec st[256];
    static_assert(sizeof(st) % 16 == 0, "the staged tile is whole 16-byte words");
    for (int64_t t0 = (int64_t)blockIdx.x * 256; t0 < n; t0 += (int64_t)gridDim.x * 256) {
        const int64_t j = t0 + threadIdx.x;
        if (j < n) {
            const int64_t p = idx ? (int64_t)idx[j] : j;
            EventRec e;
            e.parn = P.parn[p]; e.pann = P.pann[p]; e.modn = P.modn[p]; e.cryn = P.cryn[p];
            e.siten = site[p];
            e.eventid = P.eventid[p];
            e.t = P.t[p];
            e.E = Eb[p]; e.x = xb[p]; e.y = yb[p]; e.z = zb[p];
            st[threadIdx.x] = e;
            if (flags) flags[j] = (P.meta[p] & 0x80u) ? 1 : 0;
        }
        __syncthreads();
        const int64_t cnt = n - t0 < 256 ? n - t0 : 256;
        const int words = (int)cnt * (int)(sizeof(EventRec) / 16);
        const uint4* w = reinterpret_cast<const uint4*>(st);
        for (int k = threadIdx.x; k < words; k += 256) out[t0 * (int64_t)(sizeof(EventRec) / 16) + k] = w[k];
        __syncthreads();
    }
}

int gather_events_mapped(const PulseDev& P, const uint32_t* idx, int64_t n, const DigiScratch& D, EventRec* out,
                         uint8_t* flags, cudaStream_t s, unsigned max_blocks)
{
    if (n <= 0) return 0;
    if (reinterpret_cast<uintptr_t>(out) & 15) return GPET_ERR_ARG;
    unsigned g = grid_for_g(n);
    if (max_blocks && g > max_blocks) g = max_blocks;
    k_gather_events_mapped<<<g, 256, 0, s>>>(P, idx, n, D.Eb, D.xb, D.yb, D.zb, D.site,
                                                         reinterpret_cast<uint4*>(out), flags);
    return cudaGetLastError() == cudaSuccess ? 0 : GPET_ERR_CUDA;
}

int gather_events(const PulseDev& P, const uint32_t* idx, int64_t n, bool blurred, const DigiScratch& D,
                  EventRec* out, uint8_t* meta, cudaStream_t s)
{
    if (n <= 0) return 0;
    k_gather_events<<<grid_for_g(n), 256, 0, s>>>(P, idx, n, blurred ? 1 : 0, D.Eb, D.xb, D.yb, D.zb, D.site, out,
                                                  meta);
    return cudaGetLastError() == cudaSuccess ? 0 : GPET_ERR_CUDA;
}

static unsigned grid_for(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 64) b = 152 * 64;
    return (unsigned)b;
}

static int ensure(void** p, size_t bytes, size_t* have)
{
    if (*have >= bytes && *p) return 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) return GPET_ERR_CUDA;
    *have = bytes;
    return 0;
}

int noise_count(const NoiseParams& np, DigiScratch& D, cudaStream_t s, int64_t* launches, int64_t* total_out)
{
    *total_out = 0;
    if (np.nint <= 0) return 0;
    if (np.nint > D.cap) return GPET_ERR_CAPACITY;
    k_noise_count<<<grid_for(np.nint, 256), 256, 0, s>>>(np, D.sel);
    ++*launches;
    uint32_t* total = reinterpret_cast<uint32_t*>(D.dcount + 6);
    scan_exclusive(D.sel, D.wcount, np.nint, D.scan_aux, total, s, launches);
    uint32_t h = 0;
    cudaMemcpyAsync(&h, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) return GPET_ERR_CUDA;
    *total_out = h;
    return 0;
}

int noise_write(const NoiseParams& np, const DigiScratch& D, const PulseDev& P, int64_t base, Counters* cnt,
                cudaStream_t s, int64_t* launches)
{
    if (np.nint <= 0) return 0;
    k_noise_write<<<grid_for(np.nint, 256), 256, 0, s>>>(np, D.wcount, P, base, cnt);
    ++*launches;
    return cudaGetLastError() == cudaSuccess ? 0 : GPET_ERR_CUDA;
}

// ---------------------------------------------------------------- sinogram
__device__ __forceinline__ void global_pos(const float* Pn, float x, float y, float z, double g[3])
{
    for (int k = 0; k < 3; ++k)
        g[k] = (double)Pn[15 + k] + (double)x * (double)Pn[21 + k] + (double)y * (double)Pn[24 + k] +
               (double)z * (double)Pn[27 + k];
}

__global__ void k_sinogram(const int64_t* __restrict__ pairs, const uint8_t* __restrict__ klass, int64_t c0,
                           int64_t nc, const uint32_t* __restrict__ single_idx, const float* __restrict__ xb,
                           const float* __restrict__ yb, const float* __restrict__ zb, const int32_t* __restrict__ pann,
                           const float* __restrict__ panels, const int32_t* __restrict__ id2panel, int32_t nid,
                           SinoParams sp, uint32_t* hist)
{
    const double kPi = 3.14159265358979323846;
    for (int64_t c = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < c0 + nc;
         c += (int64_t)gridDim.x * blockDim.x) {
        if (!((sp.class_mask >> klass[c]) & 1)) continue;
        double g[2][3];
        bool ok = true;
        for (int e = 0; e < 2; ++e) {
            const uint32_t p = single_idx[pairs[2 * c + e]];
            const int id = pann[p];
            const int pi = (id >= 0 && id < nid) ? id2panel[id] : -1;
            if (pi < 0) { ok = false; break; }
            global_pos(panels + pi * kPanelStride, xb[p], yb[p], zb[p], g[e]);
        }
        if (!ok) continue;
        const double dx = g[1][0] - g[0][0], dy = g[1][1] - g[0][1];
        const double len = sqrt(dx * dx + dy * dy);
        if (!(len > 0.0)) continue;
        double phi = atan2(dy, dx);
        double sd = (g[0][0] * -dy + g[0][1] * dx) / len;
        if (phi < 0.0) { phi += kPi; sd = -sd; }
        if (phi >= kPi) { phi -= kPi; sd = -sd; }
        const double z = 0.5 * (g[0][2] + g[1][2]);
        const double fs = (sd + sp.s_max) / (2.0 * sp.s_max) * sp.n_s;
        const double fp = phi / kPi * sp.n_phi;
        const double fz = (z + sp.z_max) / (2.0 * sp.z_max) * sp.n_z;
        if (!(fs >= 0.0 && fs < sp.n_s && fz >= 0.0 && fz < sp.n_z)) continue;
        int is = (int)fs, ip = (int)fp, iz = (int)fz;
        if (ip >= sp.n_phi) ip = sp.n_phi - 1;
        atomicAdd(&hist[((int64_t)iz * sp.n_phi + ip) * sp.n_s + is], 1u);
    }
}

int sinogram_device(const int64_t* pairs, const uint8_t* klass, int64_t c0, int64_t nc, const uint32_t* single_idx,
                    const DigiScratch& D, const int32_t* pann, const float* panels, const int32_t* id2panel,
                    int32_t nid, SinoParams sp, uint32_t* hist, cudaStream_t s)
{
    if (nc <= 0) return 0;
    k_sinogram<<<grid_for(nc, 256), 256, 0, s>>>(pairs, klass, c0, nc, single_idx, D.xb, D.yb, D.zb, pann, panels,
                                                 id2panel, nid, sp, hist);
    return cudaGetLastError() == cudaSuccess ? 0 : GPET_ERR_CUDA;
}

int digitize_device(const PulseDev& P, int64_t n, const DigiParams* d_prms, int nsims, DigiScratch& D,
                    Counters* d_cnt, cudaStream_t s, int64_t* launches, int64_t* n_singles_out, int64_t* n_coinc_out)
{
    // dcount: [0] selected [2] singles (uint32, scan total) [4] scratch scan total
    // [8], [9] survivors' time range (ordered bits) [10] their largest site
    unsigned long long hc[11] = {0};
    cudaMemsetAsync(D.dcount, 0, 16 * sizeof(unsigned long long), s);
    cudaMemsetAsync(D.dcount + 8, 0xFF, sizeof(unsigned long long), s);
    const int32_t* psim = nsims > 1 ? P.sim : nullptr;
    PulseDev Pv = P;
    Pv.sim = const_cast<int32_t*>(psim);
    if (n > 0) {
        k_blur_threshold<<<grid_for(n, 256), 256, 0, s>>>(Pv, n, d_prms, D.Eb, D.xb, D.yb, D.zb, D.site, D.sel,
                                                          D.dcount + 0, D.dcount + 8);
        ++*launches;
    }
    cudaMemcpyAsync(hc, D.dcount, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return GPET_ERR_CUDA;
    const int64_t m = (int64_t)hc[0];
    uint32_t* total = reinterpret_cast<uint32_t*>(D.dcount + 4);
    int sim_bits = 0;
    while ((1 << sim_bits) < nsims) sim_bits++;
    sim_bits = (sim_bits + 7) / 8 * 8;
    // time order
    uint64_t *ka = D.key_a, *kb = D.key_b;
    uint32_t *va = D.idx_a, *vb = D.idx_b;
    if (m > 0) {
        const int tbits = launch_time_keys(D.sel, m, P.t, hc + 8, ka, va, s);
        ++*launches;
        radix_sort(ka, va, kb, vb, m, tbits, D.hist, D.scan_aux, total, s, launches);
        k_tie_fix<<<grid_for(m, 256), 256, 0, s>>>(ka, va, m, P.t, P.parn, P.meta);
        ++*launches;
        if (psim) {   // (simulation, t, parn, slot)
            k_sim_keys<<<grid_for(m, 256), 256, 0, s>>>(va, m, psim, ka, va);
            ++*launches;
            radix_sort(ka, va, kb, vb, m, sim_bits, D.hist, D.scan_aux, total, s, launches);
        }
        cudaMemcpyAsync(D.torder, va, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s);
        if (psim) {
            k_count_by_sim<<<grid_for(m, 256), 256, 0, s>>>(D.torder, m, psim, d_cnt, CF(n_thr));
        } else {   // one simulation: its count is m
            k_add_count<<<1, 1, 0, s>>>(d_cnt, CF(n_thr), (unsigned long long)m);
        }
        // site order
        const int site_bits = psim ? 32 + sim_bits : site_key_bits(hc[10]);
        k_site_keys<<<grid_for(m, 256), 256, 0, s>>>(D.torder, m, D.site, psim, ka, va);
        *launches += 2;
        radix_sort(ka, va, kb, vb, m, site_bits, D.hist, D.scan_aux, total, s, launches);
        // dead time on the site order
        k_deadtime<<<grid_for(m, 256), 256, 0, s>>>(va, ka, m, P.t, d_prms, psim ? 1 : 0, D.flags, d_cnt);
        // energy window over the time order, ordered compaction
        k_window_pred<<<grid_for(m, 256), 256, 0, s>>>(D.torder, m, D.flags, D.Eb, psim, d_prms, D.sel, d_cnt);
        *launches += 2;
        scan_exclusive(D.sel, D.wcount, m, D.scan_aux, reinterpret_cast<uint32_t*>(D.dcount + 2), s, launches);
        k_compact<<<grid_for(m, 256), 256, 0, s>>>(D.torder, D.sel, D.wcount, m, D.single_idx);
        ++*launches;
    }
    cudaMemcpyAsync(hc, D.dcount, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return GPET_ERR_CUDA;
    const int64_t ns = m > 0 ? (int64_t)(uint32_t)(hc[2] & 0xffffffffull) : 0;
    // coincidences
    int64_t nc = 0;
    if (ns > 0) {
        cudaMemsetAsync(D.wcount, 0, sizeof(uint32_t) * ns, s);
        cudaMemsetAsync(D.wend, 0, sizeof(uint32_t) * ns, s);
        k_coinc_count<<<grid_for(ns, 256), 256, 0, s>>>(D.single_idx, ns, P.t, P.pann, psim, d_prms, D.wcount, D.wend,
                                                        d_cnt);
        ++*launches;
        scan_exclusive(D.wcount, D.sel, ns, D.scan_aux, total, s, launches);
        uint32_t hn = 0;
        cudaMemcpyAsync(&hn, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return GPET_ERR_CUDA;
        nc = hn;
        if (nc > D.coinc_cap) {
            cudaFree(D.coinc_pairs);
            cudaFree(D.coinc_class);
            D.coinc_pairs = nullptr; D.coinc_class = nullptr;
            int64_t cap = nc + nc / 4 + 1024;
            if (cudaMalloc(&D.coinc_pairs, sizeof(int64_t) * 2 * cap) != cudaSuccess ||
                cudaMalloc(&D.coinc_class, cap) != cudaSuccess) {
                D.coinc_cap = 0;
                return GPET_ERR_CUDA;
            }
            D.coinc_cap = cap;
        }
        k_coinc_write<<<grid_for(ns, 256), 256, 0, s>>>(D.single_idx, ns, D.wend, D.sel, P.pann, P.eventid, P.meta,
                                                        psim, d_prms, D.coinc_pairs, D.coinc_class, D.coinc_cap,
                                                        d_cnt);
        ++*launches;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return GPET_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return GPET_ERR_CUDA;
    *n_singles_out = ns;
    *n_coinc_out = nc;
    return 0;
}

}  // namespace gpet
