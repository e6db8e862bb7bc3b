// surrogate.cu - the learned detector response (a new stage; the reference
// always transports photons through the panels, gPET_kernals.cu:839-1233).
//
// Model: 16 inputs (entry point y, z in the panel, direction, energy, an
// 8-wide learned panel embedding, the entry point's offset from the centre of
// its crystal in y and z in pitches) -> 4 x 256 SiLU -> 204
// outputs (two sets of 64 crystal logits, one per class of deposited energy,
// a 4-component Gaussian mixture over the depth of the pulse, 64 logits of the
// deposited-energy fraction; padded to 208). The crystal is drawn given the
// energy bin: from the first set below bin kClassBin, else from the second.
// BF16 weights and activations, FP32 accumulation in tensor memory.
//
//   k_mlp_fwd<train>  fused forward: one CTA of 512 threads per 128 samples
//                     (a tile; CTAs are persistent over tiles);
//                     activations stay in shared memory, each layer's weight
//                     image arrives by bulk copy (the next one while the
//                     current layer's epilogue runs), tcgen05.mma into TMEM,
//                     epilogue (bias, SiLU, bf16) back into shared memory.
//                     train: saves pre-activations and activations; else:
//                     samples the response and appends pulses.
//   k_umma_gemm       D (+)= A * B^T from strided global operands, split over
//                     K: the backward products dH = dZ W and dW = dZ^T H.
//   elementwise       features, loss and output gradient, SiLU backward,
//                     bias and embedding gradients, Adam, weight images.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "surrogate.h"
#include "umma.cuh"
#include "../../include/gpet.h"
#include "../../include/gpet_surrogate.h"

namespace gpet {

constexpr uint32_t kWaitLimit = 1u << 24;   // mbarrier polls before a wait gives up
constexpr uint32_t kTagSurrogate = 6;       // stream tag of the surrogate's draws

namespace sg {
constexpr int kIn = 16, kFeat = 16, kHid = 256, kOut = 208, kOutUsed = 204, kEmb = 6;
constexpr int kEmbCol = 8;   // first input column of the panel embedding
constexpr int kCry = 64, kMix = 4, kBins = 64;
constexpr int kClassBin = 40;   // energy bins >= this (deposit >= 62.5 % of E) take the second crystal set
constexpr int kColW = 128, kColMu = 132, kColLs = 136, kColE = 140;
constexpr int kLayers = 5;
constexpr float kLsMin = -7.0f, kLsMax = 3.0f;   // log sigma of a mixture component, clamped
__host__ __device__ constexpr int fan_in(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int fan_out(int l) { return l == kLayers - 1 ? kOut : kHid; }
__host__ __device__ constexpr int64_t w_off(int l)
{
    int64_t o = 0;
    for (int i = 0; i < l; ++i) o += (int64_t)fan_out(i) * fan_in(i) + fan_out(i);
    return o;
}
__host__ __device__ constexpr int64_t b_off(int l) { return w_off(l) + (int64_t)fan_out(l) * fan_in(l); }
constexpr int64_t kEmbOff = w_off(kLayers);
__host__ __device__ constexpr uint32_t img_off(int l)
{
    uint32_t o = 0;
    for (int i = 0; i < l; ++i) o += (uint32_t)(fan_out(i) * fan_in(i) * 2);
    return o;
}
constexpr uint32_t kImgBytes = img_off(kLayers);
constexpr uint32_t kSmemA = 128 * kHid * 2;   // activations of 128 samples
constexpr uint32_t kSmemB = kHid * kHid * 2;  // one weight image
static_assert(kSmemB >= (uint32_t)kOut * kHid * 2, "head image fits");
}  // namespace sg

// forward SiLU with the fast exponential and reciprocal: its result is
// rounded to bf16 next
__device__ __forceinline__ float silu(float z) { return z * __frcp_rn(1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat16 x = __float2bfloat16_rn(a), y = __float2bfloat16_rn(b);
    return (uint32_t)__bfloat16_as_ushort(x) | ((uint32_t)__bfloat16_as_ushort(y) << 16);
}

// 16 features of a photon entering a panel: y, z over the half-widths,
// direction, E / 511 keV; where its straight path is at half the panel depth
// and where it enters, each as the offset from the centre of the crystal it is
// in (-0.5 .. 0.5 pitch: the crystal becomes a linear function of the inputs);
// the panel's learned embedding
__device__ __forceinline__ void features(const SurrogateDev& sd, const float* __restrict__ emb, int panel, float y,
                                         float z, float ux, float uy, float uz, float E, float f[16])
{
    f[0] = y / sd.half_y;
    f[1] = z / sd.half_z;
    f[2] = ux;
    f[3] = uy;
    f[4] = uz;
    f[5] = E * (1.0f / 511000.0f);
    const float a = fmaxf(fabsf(ux), 0.05f), hd = 0.5f * sd.depth;
    const float ym = y + uy / a * hd, zm = z + uz / a * hd;
    const float tym = (ym + sd.half_y) / sd.cry_pitch_y, tzm = (zm + sd.half_z) / sd.cry_pitch_z;
    f[6] = tym - floorf(tym) - 0.5f;
    f[7] = tzm - floorf(tzm) - 0.5f;
    for (int k = 0; k < sg::kEmb; ++k) f[sg::kEmbCol + k] = emb[panel * sg::kEmb + k];
    const float ty = (y + sd.half_y) / sd.cry_pitch_y, tz = (z + sd.half_z) / sd.cry_pitch_z;
    f[14] = ty - floorf(ty) - 0.5f;
    f[15] = tz - floorf(tz) - 0.5f;
}

// ---------------------------------------------------------------- self-test
// D[128 x N] = A[128 x K] * B[N x K]^T for one CTA of 128 threads: A and B
// row-major bf16 in global memory, D row-major f32. K a multiple of 16 up to
// 256, N a multiple of 16 up to 256.
__global__ void __launch_bounds__(128) k_umma_selftest(const __nv_bfloat16* __restrict__ A,
                                                       const __nv_bfloat16* __restrict__ B, int K, int N, float* D,
                                                       int* err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    unsigned char* sA = sm;
    unsigned char* sB = sm + 128 * K * 2;
    for (int i = threadIdx.x; i < 128 * K; i += 128)
        *reinterpret_cast<__nv_bfloat16*>(sA + umma::img_offset(i / K, i % K, 128)) = A[i];
    for (int i = threadIdx.x; i < N * K; i += 128)
        *reinterpret_cast<__nv_bfloat16*>(sB + umma::img_offset(i / K, i % K, N)) = B[i];
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(&tbase, 256);
        umma::tmem_relinquish();
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tbase;
    if (threadIdx.x == 0) {
        const uint32_t idesc = umma::idesc_bf16_f32(128, (uint32_t)N);
        for (int ks = 0; ks < K / 16; ++ks) {
            const uint64_t ad = umma::smem_desc(umma::smem_u32(sA) + ks * 2 * 128 * 16, 128 * 16, 128);
            const uint64_t bd = umma::smem_desc(umma::smem_u32(sB) + ks * 2 * N * 16, (uint32_t)N * 16, 128);
            umma::mma_bf16(tmem, ad, bd, idesc, ks > 0);
        }
        umma::mma_commit(&bar);
    }
    const bool ok = __syncthreads_and(umma::mbar_wait(&bar, 0, kWaitLimit));
    umma::fence_after_sync();
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(err, 1);
    } else {
        const uint32_t row = 32 * warp + (threadIdx.x & 31);
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
        for (int c = 0; c < N; c += 32) {
            float v[32];
            umma::tmem_ld32(taddr + c, v);
            for (int j = 0; j < 32 && c + j < N; ++j) D[row * N + c + j] = v[j];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------- forward
struct FwdTrain {
    const __nv_bfloat16* X;       // [n][16]
    int64_t n;
    float* Z;                     // [4][n][256] pre-activations of the hidden layers
    __nv_bfloat16* H;             // [4][n][256] their bf16 activations
    float* out;                   // [n][144]
};

struct FwdInfer {
    QueueDev q;
    const uint32_t* sidx;
    const unsigned long long* scount;
    const SimDesc* sims;
    PulseDev P;
    Counters* cnt;
};

// a warp's 32 TMEM lanes, columns [c0, c0 + 32): all lanes must call it
__device__ __forceinline__ void ld_cols(uint32_t taddr, int c0, float (&v)[32]) { umma::tmem_ld32(taddr + c0, v); }

__device__ __forceinline__ float tanh_approx(float x)
{
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The response of a photon is sampled from the head's outputs in TMEM by
// three warp groups at once (each thread: one row of the tile): the deposited
// energy bin, the crystal, the depth. Each draws from the photon's own stream
// (tag 6, id = parn) in the fixed order ue, uw, uc, um, zn, skipping
// the draws of the others. hb: the head's bias.

// deposited-energy fraction bin: softmax over columns [140, 204)
__device__ __forceinline__ int sample_energy(uint32_t taddr, const float* hb, float ue)
{
    using namespace sg;
    static_assert(kColE >= 128 && kColE + kBins <= 208, "energy columns within the three loads");
    uint32_t a[32], b[32], c[16];
    umma::tmem_ld32_nowait(taddr + 128, a);
    umma::tmem_ld32_nowait(taddr + 160, b);
    umma::tmem_ld16_nowait(taddr + 192, c);
    umma::tmem_wait_ld();
    float e[kBins];
#pragma unroll
    for (int k = 0; k < kBins; ++k) {
        const int col = kColE + k;
        const uint32_t raw = col < 160 ? a[col - 128] : (col < 192 ? b[col - 160] : c[col - 192]);
        e[k] = __uint_as_float(raw) + hb[col];
    }
    float mx = -1e30f;
#pragma unroll
    for (int k = 0; k < kBins; ++k) mx = fmaxf(mx, e[k]);
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < kBins; ++k) {
        e[k] = __expf(e[k] - mx);
        sum += e[k];
    }
    const float target = ue * sum;
    float acc = 0.0f;
    int bin = kBins - 1;
    bool found = false;
#pragma unroll
    for (int k = 0; k < kBins; ++k) {
        if (!found) {
            acc += e[k];
            if (acc >= target) { bin = k; found = true; }
        }
    }
    return bin;
}

// index drawn with probability softmax(v[0..n)) at uniform u (first index
// whose running sum reaches u times the total)
template <int N>
__device__ __forceinline__ int softmax_draw(float (&v)[N], int n, float u)
{
    float mx = -1e30f;
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (k < n) mx = fmaxf(mx, v[k]);
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k < n) {
            v[k] = __expf(v[k] - mx);
            sum += v[k];
        }
    }
    const float target = u * sum;
    float acc = 0.0f;
    int pick = n - 1;
    bool found = false;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        if (k < n && !found) {
            acc += v[k];
            if (acc >= target) { pick = k; found = true; }
        }
    }
    return pick;
}

// crystal of set `set` (columns [64 set, 64 set + 64)): one softmax over the
// ncry crystals, or (fact) from the joint of a row softmax (the first 32
// columns, ny rows) and a column softmax (the last 32, nz columns) weighted
// per cell by W[row * 32 + column]: the row first (uniform uc) from its
// marginal, then the column given the row (uc2)
__device__ __forceinline__ int sample_crystal(uint32_t taddr, const float* hb, int set, int ncry, int fact, int ny,
                                              int nz, const float* __restrict__ W, float uc, float uc2)
{
    using namespace sg;
    const int c0 = kCry * set;
    uint32_t a[32], b[32];
    umma::tmem_ld32_nowait(taddr + c0, a);
    umma::tmem_ld32_nowait(taddr + c0 + 32, b);
    umma::tmem_wait_ld();
    if (fact) {
        float r[32], c[32];
        float mr = -1e30f, mc = -1e30f;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            r[k] = __uint_as_float(a[k]) + hb[c0 + k];
            c[k] = __uint_as_float(b[k]) + hb[c0 + 32 + k];
            if (k < ny) mr = fmaxf(mr, r[k]);
            if (k < nz) mc = fmaxf(mc, c[k]);
        }
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            c[k] = k < nz ? __expf(c[k] - mc) : 0.0f;
            r[k] = k < ny ? __expf(r[k] - mr) : 0.0f;
        }
        const float* w = W + set * 1024;
        // row marginal: p(row) sum over columns of p(column) W
        float tot = 0.0f;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            if (k < ny) {
                float srow = 0.0f;
                for (int j = 0; j < nz; ++j) srow = fmaf(c[j], __ldg(w + k * 32 + j), srow);
                r[k] *= srow;
                tot += r[k];
            }
        }
        int ly = ny - 1;
        {
            const float target = uc * tot;
            float acc = 0.0f;
            bool found = false;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
                if (k < ny && !found) {
                    acc += r[k];
                    if (acc >= target) { ly = k; found = true; }
                }
            }
        }
        // the column given the row
        float ct = 0.0f;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            if (k < nz) {
                c[k] *= __ldg(w + ly * 32 + k);
                ct += c[k];
            }
        }
        int lz = nz - 1;
        {
            const float target = uc2 * ct;
            float acc = 0.0f;
            bool found = false;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
                if (k < nz && !found) {
                    acc += c[k];
                    if (acc >= target) { lz = k; found = true; }
                }
            }
        }
        return ly + ny * lz;
    }
    float e[kCry];
#pragma unroll
    for (int k = 0; k < kCry; ++k) e[k] = __uint_as_float(k < 32 ? a[k] : b[k - 32]) + hb[c0 + k];
    return softmax_draw(e, ncry, uc);
}

// depth below the entry face over the panel depth: one component of the
// Gaussian mixture in columns [128, 140), clamped to [0, 1]
__device__ __forceinline__ float sample_depth(uint32_t taddr, const float* hb, float um, float zn)
{
    using namespace sg;
    static_assert(kColW == 128 && kColLs + kMix <= 144, "mixture columns within one load");
    uint32_t a[16];
    umma::tmem_ld16_nowait(taddr + 128, a);
    umma::tmem_wait_ld();
    float w[kMix];
    float wm = -1e30f;
#pragma unroll
    for (int k = 0; k < kMix; ++k) {
        w[k] = __uint_as_float(a[kColW - 128 + k]) + hb[kColW + k];
        wm = fmaxf(wm, w[k]);
    }
    float ws = 0.0f;
#pragma unroll
    for (int k = 0; k < kMix; ++k) {
        w[k] = __expf(w[k] - wm);
        ws += w[k];
    }
    int comp = kMix - 1;
    float acc = 0.0f;
    bool found = false;
#pragma unroll
    for (int k = 0; k < kMix; ++k) {
        if (!found) {
            acc += w[k];
            if (acc >= um * ws) { comp = k; found = true; }
        }
    }
    float mu = 0.0f, ls = 0.0f;
#pragma unroll
    for (int k = 0; k < kMix; ++k)
        if (k == comp) {
            mu = __uint_as_float(a[kColMu - 128 + k]) + hb[kColMu + k];
            ls = __uint_as_float(a[kColLs - 128 + k]) + hb[kColLs + k];
        }
    ls = fminf(fmaxf(ls, kLsMin), kLsMax);
    return fminf(fmaxf(mu + __expf(ls) * zn, 0.0f), 1.0f);
}

// append the photon's pulse (deposit bin > 0), one atomic per warp
__device__ __forceinline__ void append_pulse(const SurrogateDev& sd, const FwdInfer& in, bool valid, int sim,
                                             int panel, int parn, int eid, int scat, float E, float ux, double t0,
                                             int bin, int cry, float depth_n, float uw, int lane)
{
    using namespace sg;
    const SimDesc& S = in.sims[valid ? sim : 0];
    const bool pulse = valid && bin > 0;
    const float Edep = bin == kBins - 1 ? E : ((float)bin + uw) * (1.0f / kBins) * E;
    const unsigned m = __ballot_sync(0xffffffffu, pulse);
    unsigned long long base = 0;
    if (m) {
        const int leader = __ffs(m) - 1;
        if (lane == leader) base = atomicAdd(in.P.count, (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    if (pulse) {
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        const unsigned long long o = base + __popc(m & lt);
        if (o < (unsigned long long)in.P.cap) {
            const float* Pn = S.panels + panel * kPanelStride;
            const int32_t pann = (int32_t)Pn[30];
            const int depth = S.rpolicy == 1 ? 2 : S.rdepth;
            const int ly = cry % sd.crystalNy, lz = cry / sd.crystalNy;
            const float dcm = depth_n * sd.depth;
            in.P.parn[o] = parn;
            in.P.pann[o] = pann;
            in.P.modn[o] = 0;
            in.P.cryn[o] = cry;
            in.P.siten[o] = depth == 0 ? 0 : (depth == 1 ? pann : pann * S.moduleN);
            in.P.eventid[o] = eid;
            in.P.t[o] = t0 + (double)(dcm / fmaxf(fabsf(ux), 1e-6f) * DM_INV_SPEED);
            in.P.E[o] = Edep;
            in.P.x[o] = dcm * sd.dirsign;
            in.P.y[o] = -sd.half_y + (float)ly * sd.cry_pitch_y + 0.5f * sd.cry_y;
            in.P.z[o] = -sd.half_z + (float)lz * sd.cry_pitch_z + 0.5f * sd.cry_z;
            in.P.meta[o] = (uint8_t)(scat ? 0x80 : 0);
            if (in.P.sim) in.P.sim[o] = sim;
        } else {
            atomicAdd(&in.cnt->pulse_drop, 1ull);
        }
    }
    add_by_sim(in.cnt, valid ? sim : 0, CF(n_pulse), pulse ? 1u : 0u);
    add_by_sim(in.cnt, valid ? sim : 0, CF(n_surrogate), valid ? 1u : 0u);
}

// threads: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows of the tile)
// and handles column quarter w / 4 of each layer's epilogue; warps 0-3 (one
// thread per row) build the inputs and sample the outputs
constexpr int kFwdThreads = 512;

template <bool kTrain>
__global__ void __launch_bounds__(kFwdThreads, 1) k_mlp_fwd(SurrogateDev sd, FwdTrain tr, FwdInfer in, int* err)
{
    using namespace sg;
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* sA = sm;
    unsigned char* sB = sm + kSmemA;
    __shared__ __align__(8) uint64_t bar_ld, bar_mma;
    __shared__ uint32_t tbase;
    // biases: hidden layers (halved for the tanh form of SiLU in inference), then the head
    __shared__ float sbias[(kLayers - 1) * kHid + kOut];
    // per tile (inference): the photon's stream and simulation, its sampled response
    __shared__ int32_t s_parn[128], s_sim[128], s_bin[128], s_cry[2][128];
    __shared__ float s_depth[128];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t n;
    if (kTrain) {
        n = tr.n;
    } else {
        unsigned long long c = *in.scount;
        n = (int64_t)(c < (unsigned long long)in.q.cap ? c : (unsigned long long)in.q.cap);
    }
    if ((int64_t)blockIdx.x * 128 >= n) return;   // the whole CTA, before any barrier or allocation
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar_ld, 1);
        umma::mbar_init(&bar_mma, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(&tbase, 256);
        umma::tmem_relinquish();
    }
    for (int i = threadIdx.x; i < (kLayers - 1) * kHid + kOut; i += blockDim.x) {
        const int l = i < (kLayers - 1) * kHid ? i / kHid : kLayers - 1;
        const int col = i - l * kHid;
        const float b = sd.params[b_off(l) + col];
        sbias[i] = (!kTrain && l < kLayers - 1) ? 0.5f * b : b;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tbase;
    const int quarter = warp & 3, cq = warp >> 2;
    const int rloc = 32 * quarter + lane;          // row of the tile this thread reads from TMEM
    const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16);
    uint32_t n_ld = 0, n_mma = 0;   // completed phases of the two barriers
    bool ok = true;
    // persistent over tiles of 128 samples
    for (int64_t row0 = (int64_t)blockIdx.x * 128; row0 < n && ok; row0 += (int64_t)gridDim.x * 128) {
        const int64_t row = row0 + rloc;
        const bool valid = row < n;
        if (threadIdx.x == 0) {
            umma::mbar_expect_tx(&bar_ld, (uint32_t)(fan_out(0) * fan_in(0) * 2));
            umma::bulk_g2s(sB, sd.img + img_off(0), (uint32_t)(fan_out(0) * fan_in(0) * 2), &bar_ld);
        }
        // the photon (inference) and its features
        float f[16];
        int sim = 0, panel = 0, parn = 0, eid = 0, scat = 0;
        float E = 0.0f, ux = 0.0f;
        double t0 = 0.0;
        for (int k = 0; k < 16; ++k) f[k] = 0.0f;
        if (cq != 0) {
            // warps 4-15 only run the epilogues
        } else if (kTrain) {
            if (valid) {
                const uint4* x = reinterpret_cast<const uint4*>(tr.X + row * kIn);
                const uint4 a = x[0], b = x[1];
                const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
                for (int k = 0; k < 8; ++k) {
                    f[2 * k] = __uint_as_float(w[k] << 16);
                    f[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
                }
            }
        } else if (valid) {
            const int64_t j = in.sidx[row];
            const int64_t cap = in.q.cap;
            const float y = in.q.f[1 * cap + j], z = in.q.f[2 * cap + j];
            ux = in.q.f[3 * cap + j];
            const float uy = in.q.f[4 * cap + j], uz = in.q.f[5 * cap + j];
            E = in.q.f[6 * cap + j];
            t0 = in.q.t[j];
            panel = in.q.i[0 * cap + j];
            parn = in.q.i[1 * cap + j];
            eid = in.q.i[2 * cap + j];
            scat = in.q.i[3 * cap + j];
            sim = in.q.i[4 * cap + j];
            features(sd, sd.params + kEmbOff, panel, y, z, ux, uy, uz, E, f);
        }
        if (!kTrain && cq == 0) {
            s_parn[rloc] = parn;
            s_sim[rloc] = sim;
        }
        if (cq == 0) {
            uint4 a, b;
            a.x = pack_bf16(f[0], f[1]); a.y = pack_bf16(f[2], f[3]); a.z = pack_bf16(f[4], f[5]);
            a.w = pack_bf16(f[6], f[7]);
            b.x = pack_bf16(f[8], f[9]); b.y = pack_bf16(f[10], f[11]); b.z = pack_bf16(f[12], f[13]);
            b.w = pack_bf16(f[14], f[15]);
            *reinterpret_cast<uint4*>(sA + umma::img_offset(rloc, 0, 128)) = a;
            *reinterpret_cast<uint4*>(sA + umma::img_offset(rloc, 8, 128)) = b;
        }
        umma::fence_proxy_async();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        for (int l = 0; l < kLayers; ++l) {
            const int K = fan_in(l), N = fan_out(l);
            ok = __syncthreads_and(umma::mbar_wait(&bar_ld, n_ld & 1u, kWaitLimit));
            n_ld++;
            if (!ok) break;
            if (threadIdx.x == 0) {
                umma::fence_after_sync();
                const uint32_t idesc = umma::idesc_bf16_f32(128, (uint32_t)N);
                for (int ks = 0; ks < K / 16; ++ks) {
                    const uint64_t ad = umma::smem_desc(umma::smem_u32(sA) + ks * 2 * 128 * 16, 128 * 16, 128);
                    const uint64_t bd =
                        umma::smem_desc(umma::smem_u32(sB) + ks * 2 * N * 16, (uint32_t)N * 16, 128);
                    umma::mma_bf16(tmem, ad, bd, idesc, ks > 0);
                }
                umma::mma_commit(&bar_mma);
            }
            ok = __syncthreads_and(umma::mbar_wait(&bar_mma, n_mma & 1u, kWaitLimit));
            n_mma++;
            umma::fence_after_sync();
            if (!ok) break;
            // the weight buffer is free: the next layer's image arrives during the epilogue
            if (threadIdx.x == 0 && l + 1 < kLayers) {
                const uint32_t bytes = (uint32_t)(fan_out(l + 1) * fan_in(l + 1) * 2);
                umma::mbar_expect_tx(&bar_ld, bytes);
                for (uint32_t o = 0; o < bytes; o += 32768u)
                    umma::bulk_g2s(sB + o, sd.img + img_off(l + 1) + o, bytes - o < 32768u ? bytes - o : 32768u,
                                   &bar_ld);
            }
            const float* bias = sbias + l * kHid;
            if (l + 1 < kLayers) {
                // this thread's 64 columns of its row: bias, SiLU, bf16, into the next layer's operand
                const int c0 = 64 * cq;
                uint32_t r0[32], r1[32];
                umma::tmem_ld32_nowait(taddr + c0, r0);
                umma::tmem_ld32_nowait(taddr + c0 + 32, r1);
                umma::tmem_wait_ld();
                auto chunk = [&](const uint32_t (&rr)[32], int c) {
                    uint32_t hp[16];
#pragma unroll
                    for (int j = 0; j < 32; j += 2) {
                        const float v0 = __uint_as_float(rr[j]), v1 = __uint_as_float(rr[j + 1]);
                        float a0, a1;
                        if (kTrain) {
                            const float z0 = v0 + bias[c + j], z1 = v1 + bias[c + j + 1];
                            if (valid) {
                                float* zr = tr.Z + ((int64_t)l * tr.n + row) * kHid + c + j;
                                zr[0] = z0;
                                zr[1] = z1;
                            }
                            a0 = silu(z0);
                            a1 = silu(z1);
                        } else {
                            // z silu(z) = h + h tanh(h), h = z / 2 (bias already halved)
                            const float h0 = fmaf(v0, 0.5f, bias[c + j]), h1 = fmaf(v1, 0.5f, bias[c + j + 1]);
                            a0 = fmaf(h0, tanh_approx(h0), h0);
                            a1 = fmaf(h1, tanh_approx(h1), h1);
                        }
                        hp[j / 2] = pack_bf16(a0, a1);
                    }
                    if (kTrain && valid) {
                        uint4* dst = reinterpret_cast<uint4*>(tr.H + ((int64_t)l * tr.n + row) * kHid + c);
                        for (int q = 0; q < 4; ++q)
                            dst[q] = make_uint4(hp[4 * q], hp[4 * q + 1], hp[4 * q + 2], hp[4 * q + 3]);
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<uint4*>(sA + umma::img_offset(rloc, c + 8 * q, 128)) =
                            make_uint4(hp[4 * q], hp[4 * q + 1], hp[4 * q + 2], hp[4 * q + 3]);
                };
                chunk(r0, c0);
                chunk(r1, c0 + 32);
            } else if (kTrain) {
                // chunks of 32 columns: quarter cq takes chunks cq and cq + 4 (7 chunks)
                for (int c = 32 * cq; c < kOut; c += 128) {
                    float v[32];
                    ld_cols(taddr, c, v);
                    if (valid)
                        for (int j = 0; j < 32 && c + j < kOut; ++j) tr.out[row * kOut + c + j] = v[j] + bias[c + j];
                }
            }
            umma::fence_proxy_async();
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
        }
        if (!kTrain && ok) {
            // the four warp groups sample the response of the tile's photons at
            // once: energy bin, the crystal of each set, depth
            const int prn = s_parn[rloc];
            const SimDesc& S = in.sims[valid ? s_sim[rloc] : 0];
            const float* hb = sbias + (kLayers - 1) * kHid;
            Stream st;
            st_init(st, S.key0, S.key1, kTagSurrogate, (uint64_t)(uint32_t)prn);
            const float ue = st_u(st), uw = st_u(st), uc = st_u(st), um = st_u(st);
            if (cq == 0) {
                s_bin[rloc] = sample_energy(taddr, hb, ue);
            } else if (cq == 1 || cq == 3) {
                // the column of a factorised head takes the stream's seventh
                // word (the depth group's normal takes the fifth and sixth)
                st_next(st);
                st_next(st);
                const float uc2 = st_u(st);
                s_cry[cq >> 1][rloc] = sample_crystal(taddr, hb, cq >> 1, sd.crystalN, sd.fact, sd.crystalNy,
                                                      sd.crystalNz, sd.corr, uc, uc2);
            } else {
                const float zn = st_normal(st);
                s_depth[rloc] = sample_depth(taddr, hb, um, zn);
            }
            umma::fence_before_sync();
            __syncthreads();
            umma::fence_after_sync();
            if (cq == 0) {
                const int bin = s_bin[rloc];
                append_pulse(sd, in, valid, sim, panel, parn, eid, scat, E, ux, t0, bin,
                             s_cry[bin >= kClassBin ? 1 : 0][rloc], s_depth[rloc], uw, lane);
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 256);
    if (!ok && threadIdx.x == 0) atomicOr(err, 1);
}

// ---------------------------------------------------------------- generic GEMM
// element (r, k) of an operand: p[r * rs + k * ks], zero outside rows x K
struct Opnd {
    const void* p;
    int32_t f32;                  // 1: float source (rounded to bf16), 0: bf16
    int64_t rs, ks, rows;
};

__device__ __forceinline__ __nv_bfloat16 opnd_at(const Opnd& o, int64_t r, int64_t k)
{
    const int64_t i = r * o.rs + k * o.ks;
    return o.f32 ? __float2bfloat16_rn(static_cast<const float*>(o.p)[i])
                 : static_cast<const __nv_bfloat16*>(o.p)[i];
}

// fill an R x 64 operand image from rows [r0, r0 + R), columns [k0, k0 + 64)
__device__ __forceinline__ void fill_image(unsigned char* img, const Opnd& o, int R, int64_t r0, int64_t k0, int64_t K)
{
    const bool kfast = o.ks == 1;
    for (int i = threadIdx.x; i < R * 64; i += blockDim.x) {
        const int r = kfast ? i / 64 : i % R;
        const int k = kfast ? i % 64 : i / R;
        const int64_t gr = r0 + r, gk = k0 + k;
        const __nv_bfloat16 v = (gr < o.rows && gk < K) ? opnd_at(o, gr, gk) : __float2bfloat16_rn(0.0f);
        *reinterpret_cast<__nv_bfloat16*>(img + umma::img_offset(r, k, R)) = v;
    }
}

// D[r][n] (+)= sum_k A(r, k) B(n, k) for rows r in [128 blockIdx.x, +128),
// n < N (a multiple of 16, <= 256), k in this CTA's split of [0, K)
__global__ void __launch_bounds__(128) k_umma_gemm(Opnd A, Opnd B, int N, int64_t K, int64_t k_per_cta, float* D,
                                                   int64_t ldd, int64_t d_rows, int atomic, int* err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* sA = sm;
    unsigned char* sB = sm + 128 * 64 * 2;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    const int warp = threadIdx.x >> 5;
    const int64_t m0 = (int64_t)blockIdx.x * 128;
    const int64_t kb = (int64_t)blockIdx.y * k_per_cta;
    const int64_t ke = kb + k_per_cta < K ? kb + k_per_cta : K;
    if (kb >= ke) return;
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(&tbase, 256);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tbase;
    bool ok = true;
    uint32_t phase = 0;
    for (int64_t kc = kb; kc < ke && ok; kc += 64, phase ^= 1u) {
        fill_image(sA, A, 128, m0, kc, ke);
        fill_image(sB, B, N, 0, kc, ke);
        umma::fence_proxy_async();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        if (threadIdx.x == 0) {
            const uint32_t idesc = umma::idesc_bf16_f32(128, (uint32_t)N);
            for (int ks = 0; ks < 4; ++ks) {
                const uint64_t ad = umma::smem_desc(umma::smem_u32(sA) + ks * 2 * 128 * 16, 128 * 16, 128);
                const uint64_t bd = umma::smem_desc(umma::smem_u32(sB) + ks * 2 * N * 16, (uint32_t)N * 16, 128);
                umma::mma_bf16(tmem, ad, bd, idesc, kc > kb || ks > 0);
            }
            umma::mma_commit(&bar);
        }
        ok = __syncthreads_and(umma::mbar_wait(&bar, phase, kWaitLimit));
        umma::fence_after_sync();
    }
    if (ok) {
        const int64_t r = m0 + 32 * warp + (threadIdx.x & 31);
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
        for (int c = 0; c < N; c += 32) {
            float v[32];
            umma::tmem_ld32(taddr + c, v);
            if (r < d_rows)
                for (int j = 0; j < 32 && c + j < N; ++j) {
                    if (atomic) atomicAdd(&D[r * ldd + c + j], v[j]);
                    else D[r * ldd + c + j] = v[j];
                }
        }
    } else if (threadIdx.x == 0) {
        atomicOr(err, 1);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------- training kernels
// features and targets of entry records; the embedding comes from params
__global__ void k_entry_features(const EntryRec* __restrict__ rec, int64_t n, SurrogateDev sd,
                                 const float* __restrict__ params, __nv_bfloat16* X, int32_t* cry, float* dep,
                                 int32_t* bin, int32_t* panel)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const EntryRec e = rec[i];
        float f[16];
        features(sd, params + sg::kEmbOff, e.panel, e.y, e.z, e.ux, e.uy, e.uz, e.E, f);
        uint4 a, b;
        a.x = pack_bf16(f[0], f[1]); a.y = pack_bf16(f[2], f[3]); a.z = pack_bf16(f[4], f[5]); a.w = pack_bf16(f[6], f[7]);
        b.x = pack_bf16(f[8], f[9]); b.y = pack_bf16(f[10], f[11]); b.z = pack_bf16(f[12], f[13]);
        b.w = pack_bf16(f[14], f[15]);
        reinterpret_cast<uint4*>(X + i * sg::kIn)[0] = a;
        reinterpret_cast<uint4*>(X + i * sg::kIn)[1] = b;
        const bool has = e.crystal >= 0 && e.Edep > 0.0f;
        cry[i] = has ? e.crystal : -1;
        dep[i] = has ? e.depth / sd.depth : 0.0f;
        int b2 = 0;
        if (has) {
            b2 = (int)(e.Edep / e.E * (float)sg::kBins);
            b2 = b2 < 1 ? 1 : (b2 > sg::kBins - 1 ? sg::kBins - 1 : b2);
        }
        bin[i] = b2;
        panel[i] = e.panel;
    }
}

// loss of each sample and d loss / d output (mean over the n samples)
// cross entropy of the logits o[0..n) against class t; d[0..n) = its gradient times scale
__device__ __forceinline__ float xent(const float* o, int n, int t, float scale, float* d)
{
    float mx = -1e30f;
    for (int k = 0; k < n; ++k) mx = fmaxf(mx, o[k]);
    float s = 0.0f;
    for (int k = 0; k < n; ++k) s += expf(o[k] - mx);
    const float lse = mx + logf(s);
    for (int k = 0; k < n; ++k) d[k] = (expf(o[k] - lse) - (k == t ? 1.0f : 0.0f)) * scale;
    return lse - o[t];
}

// fact: the crystal head is a row softmax (ny) and a column softmax (nz)
__global__ void k_loss(const float* __restrict__ out, int64_t n, const int32_t* __restrict__ cry,
                       const float* __restrict__ dep, const int32_t* __restrict__ bin, int crystalN, int fact,
                       int ny, int nz, float* dout, float* loss_sum)
{
    using namespace sg;
    __shared__ float red[8];
    const float scale = 1.0f / (float)n;
    float lsum = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* o = out + i * kOut;
        float* d = dout + i * kOut;
        for (int c = 0; c < kOut; ++c) d[c] = 0.0f;
        // energy fraction: cross entropy over 64 bins
        {
            float mx = -1e30f;
            for (int k = 0; k < kBins; ++k) mx = fmaxf(mx, o[kColE + k]);
            float s = 0.0f;
            for (int k = 0; k < kBins; ++k) s += expf(o[kColE + k] - mx);
            const float lse = mx + logf(s);
            lsum += lse - o[kColE + bin[i]];
            for (int k = 0; k < kBins; ++k)
                d[kColE + k] = (expf(o[kColE + k] - lse) - (k == bin[i] ? 1.0f : 0.0f)) * scale;
        }
        if (cry[i] >= 0) {
            // the crystal set of the sample's energy class
            const int c0 = bin[i] >= kClassBin ? kCry : 0;
            if (fact) {
                lsum += xent(o + c0, ny, cry[i] % ny, scale, d + c0);
                lsum += xent(o + c0 + 32, nz, cry[i] / ny, scale, d + c0 + 32);
            } else {
                lsum += xent(o + c0, crystalN, cry[i], scale, d + c0);
            }
            // depth: Gaussian mixture negative log likelihood
            const float x = dep[i];
            float lw[kMix], lp[kMix], ls[kMix], mu[kMix];
            float wm = -1e30f;
            for (int k = 0; k < kMix; ++k) wm = fmaxf(wm, o[kColW + k]);
            float ws = 0.0f;
            for (int k = 0; k < kMix; ++k) ws += expf(o[kColW + k] - wm);
            const float wlse = wm + logf(ws);
            float pm = -1e30f;
            for (int k = 0; k < kMix; ++k) {
                lw[k] = o[kColW + k] - wlse;
                mu[k] = o[kColMu + k];
                ls[k] = fminf(fmaxf(o[kColLs + k], kLsMin), kLsMax);
                const float zz = (x - mu[k]) * expf(-ls[k]);
                lp[k] = lw[k] - 0.5f * zz * zz - ls[k] - 0.91893853320467274f;
                pm = fmaxf(pm, lp[k]);
            }
            float ps = 0.0f;
            for (int k = 0; k < kMix; ++k) ps += expf(lp[k] - pm);
            const float plse = pm + logf(ps);
            lsum += -plse;
            for (int k = 0; k < kMix; ++k) {
                const float g = expf(lp[k] - plse);     // responsibility
                const float pw = expf(lw[k]);
                const float iv = expf(-2.0f * ls[k]);
                const float dx = x - mu[k];
                d[kColW + k] = (pw - g) * scale;
                d[kColMu + k] = -g * dx * iv * scale;
                const float raw = o[kColLs + k];
                d[kColLs + k] = (raw > kLsMin && raw < kLsMax) ? -g * (dx * dx * iv - 1.0f) * scale : 0.0f;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        atomicAdd(loss_sum, s * scale);
    }
}

// the batch's records, in the epoch's order, from the training set on the device
__global__ void k_gather_records(const EntryRec* __restrict__ all, const uint32_t* __restrict__ order, int64_t n,
                                 EntryRec* out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = all[order[i]];
}

// expected counts of a batch under the model: acc[set * kCry + crystal] of
// each (energy class, crystal) — per record the probability of the class (its
// energy-bin probabilities summed over the class's bins; bin 0 = no pulse
// belongs to neither) times the class's crystal probability — and
// acc[2 * kCry + bin] of each energy bin. One warp per record, two bins and
// two crystals per lane.
__global__ void __launch_bounds__(256) k_calib_accum(const float* __restrict__ out, int64_t n, int crystalN,
                                                     double* acc)
{
    using namespace sg;
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float a[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
    float ea[2] = {0.0f, 0.0f};
    for (int64_t i = w0; i < n; i += nw) {
        const float* o = out + i * kOut;
        const float e0 = o[kColE + lane], e1 = o[kColE + 32 + lane];
        float mx = fmaxf(e0, e1);
        for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
        const float x0 = expf(e0 - mx), x1 = expf(e1 - mx);
        const int b0 = lane, b1 = 32 + lane;
        float s = x0 + x1;
        float c0 = (b0 >= 1 && b0 < kClassBin ? x0 : 0.0f) + (b1 >= 1 && b1 < kClassBin ? x1 : 0.0f);
        float c1 = (b0 >= kClassBin ? x0 : 0.0f) + (b1 >= kClassBin ? x1 : 0.0f);
        for (int d = 16; d > 0; d >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, d);
            c0 += __shfl_xor_sync(0xffffffffu, c0, d);
            c1 += __shfl_xor_sync(0xffffffffu, c1, d);
        }
        ea[0] += x0 / s;
        ea[1] += x1 / s;
#pragma unroll
        for (int set = 0; set < 2; ++set) {
            const float* l = o + set * kCry;
            const bool v0 = lane < crystalN, v1 = 32 + lane < crystalN;
            const float l0 = v0 ? l[lane] : -1e30f, l1 = v1 ? l[32 + lane] : -1e30f;
            float m2 = fmaxf(l0, l1);
            for (int d = 16; d > 0; d >>= 1) m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, d));
            const float y0 = v0 ? expf(l0 - m2) : 0.0f, y1 = v1 ? expf(l1 - m2) : 0.0f;
            float t = y0 + y1;
            for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
            const float w = (set ? c1 : c0) / (s * t);
            a[set][0] += w * y0;
            a[set][1] += w * y1;
        }
    }
#pragma unroll
    for (int set = 0; set < 2; ++set) {
        atomicAdd(&acc[set * kCry + lane], (double)a[set][0]);
        atomicAdd(&acc[set * kCry + 32 + lane], (double)a[set][1]);
    }
    atomicAdd(&acc[2 * kCry + lane], (double)ea[0]);
    atomicAdd(&acc[2 * kCry + 32 + lane], (double)ea[1]);
}

// expected counts of a batch under a factorised head: acc[set * 1024 + row *
// 32 + column] of each (energy class, row, column) cell — the class
// probability times the cell's share of the class's joint, p(row) p(column)
// W[set][row][column] normalised — and acc[2048 + bin] of each energy bin.
// One warp per record; lane j holds column j and sums over the rows.
__global__ void __launch_bounds__(256) k_calib_accum_grid(const float* __restrict__ out, int64_t n, int ny, int nz,
                                                          const float* __restrict__ W, double* acc)
{
    using namespace sg;
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float a[2][32];
#pragma unroll
    for (int set = 0; set < 2; ++set)
#pragma unroll
        for (int k = 0; k < 32; ++k) a[set][k] = 0.0f;
    float ea[2] = {0.0f, 0.0f};
    for (int64_t i = w0; i < n; i += nw) {
        const float* o = out + i * kOut;
        const float e0 = o[kColE + lane], e1 = o[kColE + 32 + lane];
        float mx = fmaxf(e0, e1);
        for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
        const float x0 = expf(e0 - mx), x1 = expf(e1 - mx);
        const int b0 = lane, b1 = 32 + lane;
        float s = x0 + x1;
        float c0 = (b0 >= 1 && b0 < kClassBin ? x0 : 0.0f) + (b1 >= 1 && b1 < kClassBin ? x1 : 0.0f);
        float c1 = (b0 >= kClassBin ? x0 : 0.0f) + (b1 >= kClassBin ? x1 : 0.0f);
        for (int d = 16; d > 0; d >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, d);
            c0 += __shfl_xor_sync(0xffffffffu, c0, d);
            c1 += __shfl_xor_sync(0xffffffffu, c1, d);
        }
        ea[0] += x0 / s;
        ea[1] += x1 / s;
#pragma unroll
        for (int set = 0; set < 2; ++set) {
            const float* l = o + set * kCry;
            const bool vr = lane < ny, vc = lane < nz;
            const float lr = vr ? l[lane] : -1e30f, lc = vc ? l[32 + lane] : -1e30f;
            float mr = lr, mc = lc;
            for (int d = 16; d > 0; d >>= 1) {
                mr = fmaxf(mr, __shfl_xor_sync(0xffffffffu, mr, d));
                mc = fmaxf(mc, __shfl_xor_sync(0xffffffffu, mc, d));
            }
            const float pr = vr ? expf(lr - mr) : 0.0f;   // this lane's row weight
            const float pc = vc ? expf(lc - mc) : 0.0f;   // this lane's column weight
            const float* w = W + set * 1024;
            // cell (row k, column lane): p(row k) p(column lane) W
            float cell[32];
            float part = 0.0f;
#pragma unroll
            for (int k = 0; k < 32; ++k) {
                const float prk = __shfl_sync(0xffffffffu, pr, k);
                cell[k] = (k < ny && vc) ? prk * pc * __ldg(w + k * 32 + lane) : 0.0f;
                part += cell[k];
            }
            for (int d = 16; d > 0; d >>= 1) part += __shfl_xor_sync(0xffffffffu, part, d);
            const float f = (set ? c1 : c0) / (s * part);
#pragma unroll
            for (int k = 0; k < 32; ++k) a[set][k] += f * cell[k];
        }
    }
#pragma unroll
    for (int set = 0; set < 2; ++set)
#pragma unroll
        for (int k = 0; k < 32; ++k)
            if (k < ny && lane < nz) atomicAdd(&acc[set * 1024 + k * 32 + lane], (double)a[set][k]);
    atomicAdd(&acc[2048 + lane], (double)ea[0]);
    atomicAdd(&acc[2048 + 32 + lane], (double)ea[1]);
}

// dZ = dH * SiLU'(Z), in place on dH
__global__ void k_silu_back(float* dH, const float* __restrict__ Z, int64_t count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dH[i] *= silu_grad(Z[i]);
}

// column sums of a [n][cols] matrix into g (+=)
__global__ void k_colsum(const float* __restrict__ M, int64_t n, int cols, float* g)
{
    const int c = blockIdx.x;
    float s = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += M[i * cols + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        g[c] += t;
    }
}

// embedding gradient: the input gradient's columns 6..13, by panel
__global__ void k_emb_grad(const float* __restrict__ dX, const int32_t* __restrict__ panel, int64_t n, float* gemb)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * sg::kEmb;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = i / sg::kEmb;
        const int k = (int)(i % sg::kEmb);
        atomicAdd(&gemb[panel[s] * sg::kEmb + k], dX[s * sg::kIn + sg::kEmbCol + k]);
    }
}

// padding entries of the parameter vector (first-layer inputs from kFeat on,
// head outputs from kOutUsed on) stay zero
__device__ __forceinline__ bool is_pad(int64_t i)
{
    using namespace sg;
    if (i < b_off(0)) return ((i - w_off(0)) % fan_in(0)) >= kFeat;
    if (i >= w_off(kLayers - 1) && i < b_off(kLayers - 1)) return (i - w_off(kLayers - 1)) / kHid >= kOutUsed;
    if (i >= b_off(kLayers - 1) && i < kEmbOff) return (i - b_off(kLayers - 1)) >= kOutUsed;
    return false;
}

__global__ void k_adam(float* p, const float* __restrict__ g, float* m, float* v, int64_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (is_pad(i)) {
            p[i] = 0.0f;
            continue;
        }
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// bf16 copies of the weights: row-major (backward operands) and operand
// images (forward)
__global__ void k_weights(const float* __restrict__ p, __nv_bfloat16* wrow, unsigned char* img)
{
    using namespace sg;
    int64_t total = 0;
    for (int l = 0; l < kLayers; ++l) total += (int64_t)fan_out(l) * fan_in(l);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int l = 0;
        int64_t j = i;
        while (j >= (int64_t)fan_out(l) * fan_in(l)) {
            j -= (int64_t)fan_out(l) * fan_in(l);
            ++l;
        }
        const int K = fan_in(l), N = fan_out(l);
        const int o = (int)(j / K), k = (int)(j % K);
        const __nv_bfloat16 v = __float2bfloat16_rn(p[w_off(l) + j]);
        wrow[w_off(l) + j] = v;
        *reinterpret_cast<__nv_bfloat16*>(img + img_off(l) + umma::img_offset(o, k, N)) = v;
    }
}

// split the queue: photons in the validated domain -> sidx, the rest -> q2
__global__ void k_route(SurrogateDev sd, QueueDev q, QueueDev q2, uint32_t* sidx, unsigned long long* scount)
{
    unsigned long long c = *q.count;
    const int64_t n = (int64_t)(c < (unsigned long long)q.cap ? c : (unsigned long long)q.cap);
    const int lane = threadIdx.x & 31;
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = base + threadIdx.x;
        const bool valid = j < n;
        bool elig = false;
        if (valid) {
            const float y = q.f[1 * q.cap + j], z = q.f[2 * q.cap + j], E = q.f[6 * q.cap + j];
            const int panel = q.i[0 * q.cap + j];
            elig = E >= sd.e_lo && E <= sd.e_hi && fabsf(y) <= sd.half_y - sd.margin &&
                   fabsf(z) <= sd.half_z - sd.margin && panel >= 0 && panel < sd.npanels && sd.panel_ok[panel];
        }
        const unsigned ms = __ballot_sync(0xffffffffu, elig);
        if (ms) {
            unsigned long long b = 0;
            const int leader = __ffs(ms) - 1;
            if (lane == leader) b = atomicAdd(scount, (unsigned long long)__popc(ms));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (elig) sidx[b + __popc(ms & lt)] = (uint32_t)j;
        }
        const bool mc = valid && !elig;
        const unsigned mm = __ballot_sync(0xffffffffu, mc);
        if (mm) {
            unsigned long long b = 0;
            const int leader = __ffs(mm) - 1;
            if (lane == leader) b = atomicAdd(q2.count, (unsigned long long)__popc(mm));
            b = __shfl_sync(0xffffffffu, b, leader);
            const unsigned long long o = b + __popc(mm & lt);
            if (mc && o < (unsigned long long)q2.cap) {
                for (int a = 0; a < 7; ++a) q2.f[a * q2.cap + o] = q.f[a * q.cap + j];
                q2.t[o] = q.t[j];
                for (int a = 0; a < 5; ++a) q2.i[a * q2.cap + o] = q.i[a * q.cap + j];
            }
        }
    }
}

static unsigned grid_cap(int64_t n, int threads, int64_t cap)
{
    int64_t b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

static int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

cudaError_t launch_route(const SurrogateDev& sd, const QueueDev& q, int64_t max_n, const QueueDev& q2,
                         uint32_t* sidx, unsigned long long* scount, cudaStream_t s)
{
    k_route<<<grid_cap(max_n, 256, (int64_t)sm_count() * 8), 256, 0, s>>>(sd, q, q2, sidx, scount);
    return cudaGetLastError();
}

cudaError_t launch_surrogate(const SurrogateDev& sd, const SimDesc* sims, const QueueDev& q, const uint32_t* sidx,
                             const unsigned long long* scount, int64_t max_n, const PulseDev& P, Counters* cnt,
                             int* err, cudaStream_t s)
{
    const int smem = (int)(sg::kSmemA + sg::kSmemB);
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fwd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    FwdInfer in{q, sidx, scount, sims, P, cnt};
    FwdTrain tr{};
    k_mlp_fwd<false><<<grid_cap(max_n, 128, sm_count()), kFwdThreads, smem, s>>>(sd, tr, in, err);
    return cudaGetLastError();
}

}  // namespace gpet

// ---------------------------------------------------------------- host object
using namespace gpet;

namespace {

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

uint64_t splitmix(uint64_t& x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

static_assert(sizeof(gpet_entry) == sizeof(EntryRec), "entry record layouts agree");

struct gpet_surrogate {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    SurGeom geom{};
    float e_lo = 100000.0f, e_hi = 520000.0f, margin = 0.3f;
    std::vector<uint8_t> panel_ok;
    int64_t nparam = 0;
    int64_t adam_t = 0;
    Buf params, grads, adam_m, adam_v, wrow, img, panel_ok_d, errflag, loss;
    // training batch scratch
    int64_t cap = 0;
    Buf X, Z, H, out, dout, dA, dB, cry, dep, bin, pan, rec;
    // training set on the device and the epoch's visiting order
    Buf all, perm, epoch_loss;
    Buf calib;   // expected (energy class, crystal) counts of a calibration pass
    Buf corr;    // factorised head: cell weights [2][32][32] (1 until calibrated)
};

namespace {

int sfail(gpet_surrogate* s, int code, const std::string& m)
{
    if (s) s->err = m;
    return code;
}

#define SCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e__ = (call);                                                              \
        if (e__ != cudaSuccess) return sfail(s, GPET_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
    } while (0)

SurrogateDev make_view(const gpet_surrogate* s)
{
    SurrogateDev d{};
    const SurGeom& g = s->geom;
    d.params = s->params.as<float>();
    d.img = s->img.as<unsigned char>();
    d.panel_ok = s->panel_ok_d.as<uint8_t>();
    d.npanels = g.npanels;
    d.half_y = 0.5f * g.panel0[1];
    d.half_z = 0.5f * g.panel0[2];
    d.depth = g.panel0[0];
    d.dirsign = g.dirsign;
    d.e_lo = s->e_lo;
    d.e_hi = s->e_hi;
    d.margin = s->margin;
    d.crystalN = g.crystalN;
    d.crystalNy = g.crystalNy;
    d.fact = g.crystalN > sg::kCry ? 1 : 0;
    d.crystalNz = g.crystalNy > 0 ? g.crystalN / g.crystalNy : 0;
    d.corr = s->corr.as<float>();
    d.rdepth = g.rdepth;
    d.rpolicy = g.rpolicy;
    d.moduleN = g.moduleN;
    d.cry_y = g.panel0[10];
    d.cry_z = g.panel0[11];
    d.cry_pitch_y = g.panel0[10] + g.panel0[13];
    d.cry_pitch_z = g.panel0[11] + g.panel0[14];
    return d;
}

int refresh_weights(gpet_surrogate* s)
{
    k_weights<<<152 * 4, 256, 0, s->stream>>>(s->params.as<float>(), s->wrow.as<__nv_bfloat16>(),
                                             s->img.as<unsigned char>());
    SCK(cudaGetLastError());
    return GPET_OK;
}

int ensure_batch(gpet_surrogate* s, int64_t n)
{
    using namespace sg;
    if (n <= s->cap) return GPET_OK;
    const int64_t c = std::max<int64_t>(n, 1024);
    SCK(s->X.ensure((size_t)c * kIn * 2));
    SCK(s->Z.ensure((size_t)4 * c * kHid * 4));
    SCK(s->H.ensure((size_t)4 * c * kHid * 2));
    SCK(s->out.ensure((size_t)c * kOut * 4));
    SCK(s->dout.ensure((size_t)c * kOut * 4));
    SCK(s->dA.ensure((size_t)c * kHid * 4));
    SCK(s->dB.ensure((size_t)c * kHid * 4));
    SCK(s->cry.ensure((size_t)c * 4));
    SCK(s->dep.ensure((size_t)c * 4));
    SCK(s->bin.ensure((size_t)c * 4));
    SCK(s->pan.ensure((size_t)c * 4));
    SCK(s->rec.ensure((size_t)c * sizeof(EntryRec)));
    s->cap = c;
    return GPET_OK;
}

// D = A * B^T over K, strided operands; d_rows rows of D are written
// k_umma_gemm uses 48 KB of shared memory but asks for 96 KB, so that at most
// two CTAs share an SM and their TMEM (2 x 256 of 512 columns) always fits
constexpr int kGemmSmem = 96 * 1024;

int gemm(gpet_surrogate* s, const Opnd& A, int64_t m_rows, const Opnd& B, int N, int64_t K, float* D, int64_t ldd,
         bool atomic)
{
    const int smem = kGemmSmem;
    const int64_t mt = (m_rows + 127) / 128;
    int64_t splits = 1, kper = K;
    if (atomic) {
        splits = std::max<int64_t>(1, std::min<int64_t>((K + 63) / 64, std::max<int64_t>(1, 152 / mt)));
        kper = ((K + splits - 1) / splits + 63) / 64 * 64;
        splits = (K + kper - 1) / kper;
    }
    dim3 grid((unsigned)mt, (unsigned)splits);
    k_umma_gemm<<<grid, 128, smem, s->stream>>>(A, B, N, K, kper, D, ldd, m_rows, atomic ? 1 : 0,
                                                 s->errflag.as<int>());
    SCK(cudaGetLastError());
    return GPET_OK;
}

// forward + loss + backward of n samples already in s->rec; gradients into
// s->grads (zeroed here), mean loss into *loss
// Loss and gradient of the n records in s->rec. loss != NULL: the batch mean
// is returned and the stream synchronised; else the mean is added to
// *acc_dev on the device and nothing waits (a training step).
int loss_and_grad(gpet_surrogate* s, int64_t n, float* loss, float* acc_dev = nullptr)
{
    using namespace sg;
    int rc = ensure_batch(s, n);
    if (rc) return rc;
    SurrogateDev sd = make_view(s);
    cudaStream_t st = s->stream;
    const unsigned g1 = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
    k_entry_features<<<g1, 256, 0, st>>>(s->rec.as<EntryRec>(), n, sd, s->params.as<float>(), s->X.as<__nv_bfloat16>(),
                                         s->cry.as<int32_t>(), s->dep.as<float>(), s->bin.as<int32_t>(),
                                         s->pan.as<int32_t>());
    FwdTrain tr{s->X.as<__nv_bfloat16>(), n, s->Z.as<float>(), s->H.as<__nv_bfloat16>(), s->out.as<float>()};
    FwdInfer in{};
    const int smem = (int)(kSmemA + kSmemB);
    SCK(cudaFuncSetAttribute(k_mlp_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    SCK(cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
    k_mlp_fwd<true><<<grid_cap(n, 128, 152), kFwdThreads, smem, st>>>(sd, tr, in, s->errflag.as<int>());
    SCK(cudaGetLastError());
    if (!acc_dev) SCK(cudaMemsetAsync(s->loss.p, 0, 4, st));
    SCK(cudaMemsetAsync(s->grads.p, 0, (size_t)s->nparam * 4, st));
    k_loss<<<g1, 256, 0, st>>>(s->out.as<float>(), n, s->cry.as<int32_t>(), s->dep.as<float>(), s->bin.as<int32_t>(),
                               s->geom.crystalN, sd.fact, sd.crystalNy, sd.crystalNz, s->dout.as<float>(),
                               acc_dev ? acc_dev : s->loss.as<float>());
    SCK(cudaGetLastError());
    float* G = s->grads.as<float>();
    const __nv_bfloat16* Wb = s->wrow.as<__nv_bfloat16>();
    // layer by layer from the head down; dZ of layer l lives in `dz`
    float* dz = s->dout.as<float>();
    float* dh_next = s->dA.as<float>();
    float* dh_other = s->dB.as<float>();
    for (int l = kLayers - 1; l >= 0; --l) {
        const int K = fan_in(l), N = fan_out(l);
        // dW = dZ^T * input: rows N (outputs), K columns (inputs), sum over samples
        Opnd A{dz, 1, 1, N, N};
        Opnd B = l == 0 ? Opnd{s->X.as<__nv_bfloat16>(), 0, 1, kIn, K}
                        : Opnd{s->H.as<__nv_bfloat16>() + (int64_t)(l - 1) * n * kHid, 0, 1, kHid, K};
        rc = gemm(s, A, N, B, K, n, G + w_off(l), K, true);
        if (rc) return rc;
        k_colsum<<<N, 256, 0, st>>>(dz, n, N, G + b_off(l));
        SCK(cudaGetLastError());
        // dInput = dZ * W: n rows, K columns, sum over the N outputs
        Opnd Ad{dz, 1, N, 1, n};
        Opnd Bw{Wb + w_off(l), 0, 1, K, K};   // B(r = input k, c = output o) = W[o][k]
        rc = gemm(s, Ad, n, Bw, K, N, dh_next, K, false);
        if (rc) return rc;
        if (l > 0) {
            k_silu_back<<<152 * 8, 256, 0, st>>>(dh_next, s->Z.as<float>() + (int64_t)(l - 1) * n * kHid,
                                                 n * (int64_t)kHid);
            SCK(cudaGetLastError());
            dz = dh_next;
            std::swap(dh_next, dh_other);
        } else {
            k_emb_grad<<<g1, 256, 0, st>>>(dh_next, s->pan.as<int32_t>(), n, G + kEmbOff);
            SCK(cudaGetLastError());
        }
    }
    if (acc_dev) return GPET_OK;
    int herr = 0;
    SCK(cudaMemcpyAsync(&herr, s->errflag.p, 4, cudaMemcpyDeviceToHost, st));
    if (loss) SCK(cudaMemcpyAsync(loss, s->loss.p, 4, cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    if (herr) return sfail(s, GPET_ERR_CUDA, "a tensor-core wait gave up");
    return GPET_OK;
}

}  // namespace

namespace gpet {

int surrogate_view(const gpet_surrogate* s, const SurGeom& g, SurrogateDev* out, const char** why)
{
    const SurGeom& h = s->geom;
    bool same = h.device == g.device && h.npanels == g.npanels && h.moduleN == g.moduleN && h.crystalN == g.crystalN &&
                h.crystalNy == g.crystalNy && h.rdepth == g.rdepth && h.rpolicy == g.rpolicy &&
                h.dirsign == g.dirsign;
    for (int k = 0; k < 15 && same; ++k) same = h.panel0[k] == g.panel0[k];
    same = same && h.ndetmat == g.ndetmat;
    for (int k = 0; k < h.ndetmat && same; ++k) same = h.det_mat[k] == g.det_mat[k] && h.det_den[k] == g.det_den[k];
    if (!same) {
        *why = "the surrogate was made for another detector (geometry, materials or readout)";
        return GPET_ERR_ARG;
    }
    *out = make_view(s);
    return GPET_OK;
}

}  // namespace gpet

extern "C" {

int gpet_umma_selftest(int device, const uint16_t* a_bf16, const uint16_t* b_bf16, int32_t K, int32_t N,
                       float* d_out)
{
    if (!a_bf16 || !b_bf16 || !d_out || K < 16 || K > 256 || K % 16 || N < 16 || N > 256 || N % 16)
        return GPET_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return GPET_ERR_NOGPU;
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    int* dErr = nullptr;
    int rc = GPET_OK;
    const size_t smem = (size_t)(128 + N) * K * 2;
    if (cudaMalloc(&dA, 128 * K * 2) != cudaSuccess || cudaMalloc(&dB, (size_t)N * K * 2) != cudaSuccess ||
        cudaMalloc(&dD, (size_t)128 * N * 4) != cudaSuccess || cudaMalloc(&dErr, 4) != cudaSuccess) {
        rc = GPET_ERR_CUDA;
    } else {
        cudaMemcpy(dA, a_bf16, 128 * K * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, b_bf16, (size_t)N * K * 2, cudaMemcpyHostToDevice);
        cudaMemset(dD, 0, (size_t)128 * N * 4);
        cudaMemset(dErr, 0, 4);
        cudaFuncSetAttribute(k_umma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_umma_selftest<<<1, 128, smem>>>(dA, dB, K, N, dD, dErr);
        int herr = 0;
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = GPET_ERR_CUDA;
        else if (cudaMemcpy(&herr, dErr, 4, cudaMemcpyDeviceToHost) != cudaSuccess || herr) rc = GPET_ERR_CUDA;
        else if (cudaMemcpy(d_out, dD, (size_t)128 * N * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = GPET_ERR_CUDA;
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dErr);
    return rc;
}

int gpet_surrogate_create(gpet_ctx* ctx, uint64_t seed, gpet_surrogate** out)
{
    if (!ctx || !out) return GPET_ERR_ARG;
    *out = nullptr;
    SurGeom g{};
    int rc = ctx_geometry(ctx, &g);
    if (rc) return rc;
    // one pulse per photon (one module, readout depth <= 2) and a crystal head
    // that holds the crystals: up to 64 in one softmax, else a grid of up to
    // 32 x 32 as rows and columns
    const bool joint = g.crystalN >= 1 && g.crystalN <= sg::kCry;
    const bool grid = g.crystalNy >= 1 && g.crystalNy <= 32 && g.crystalN % g.crystalNy == 0 &&
                      g.crystalN / g.crystalNy <= 32;
    if (g.moduleN != 1 || !(joint || grid) || g.rdepth > 2 || g.npanels < 1) return GPET_ERR_ARG;
    if (cudaSetDevice(g.device) != cudaSuccess) return GPET_ERR_NOGPU;
    auto* s = new gpet_surrogate();
    s->device = g.device;
    s->geom = g;
    s->panel_ok.assign(g.npanels, 1);
    s->nparam = sg::kEmbOff + (int64_t)g.npanels * sg::kEmb;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return GPET_ERR_CUDA;
    }
    // initial parameters: uniform(-1/sqrt(fan in), +) weights (head x 0.1),
    // zero biases, embedding uniform(-0.1, 0.1)
    std::vector<float> p((size_t)s->nparam, 0.0f);
    uint64_t st = seed ^ 0x5851F42D4C957F2Dull;
    auto uni = [&]() { return (float)((splitmix(st) >> 11) * (1.0 / 9007199254740992.0)) * 2.0f - 1.0f; };
    for (int l = 0; l < sg::kLayers; ++l) {
        const int K = sg::fan_in(l), N = sg::fan_out(l);
        const float a = (l == sg::kLayers - 1 ? 0.1f : 1.0f) / std::sqrt((float)(l == 0 ? sg::kFeat : K));
        for (int o = 0; o < N; ++o)
            for (int k = 0; k < K; ++k) {
                const bool pad = (l == 0 && k >= sg::kFeat) || (l == sg::kLayers - 1 && o >= sg::kOutUsed);
                p[(size_t)(sg::w_off(l) + (int64_t)o * K + k)] = pad ? 0.0f : a * uni();
            }
    }
    for (int64_t i = sg::kEmbOff; i < s->nparam; ++i) p[(size_t)i] = 0.1f * uni();
    rc = GPET_OK;
    if (s->params.ensure((size_t)s->nparam * 4) || s->grads.ensure((size_t)s->nparam * 4) ||
        s->adam_m.ensure((size_t)s->nparam * 4) || s->adam_v.ensure((size_t)s->nparam * 4) ||
        s->wrow.ensure((size_t)s->nparam * 2) || s->img.ensure(sg::kImgBytes) ||
        s->panel_ok_d.ensure((size_t)g.npanels) || s->errflag.ensure(4) || s->loss.ensure(4) ||
        s->corr.ensure(2048 * 4))
        rc = GPET_ERR_CUDA;
    if (!rc) {
        const std::vector<float> ones(2048, 1.0f);
        cudaMemcpy(s->corr.p, ones.data(), ones.size() * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(s->params.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice);
        cudaMemset(s->adam_m.p, 0, (size_t)s->nparam * 4);
        cudaMemset(s->adam_v.p, 0, (size_t)s->nparam * 4);
        cudaMemset(s->errflag.p, 0, 4);
        cudaMemcpy(s->panel_ok_d.p, s->panel_ok.data(), s->panel_ok.size(), cudaMemcpyHostToDevice);
        rc = refresh_weights(s);
        if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = GPET_ERR_CUDA;
    }
    if (rc) {
        cudaStreamDestroy(s->stream);
        delete s;
        return rc;
    }
    *out = s;
    return GPET_OK;
}

void gpet_surrogate_destroy(gpet_surrogate* s)
{
    if (!s) return;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
    delete s;
}

const char* gpet_surrogate_last_error(gpet_surrogate* s) { return s ? s->err.c_str() : "null surrogate"; }

int64_t gpet_surrogate_param_count(gpet_surrogate* s) { return s ? s->nparam : -1; }

int gpet_surrogate_get_params(gpet_surrogate* s, float* out, int64_t n)
{
    if (!s || !out || n != s->nparam) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    SCK(cudaMemcpy(out, s->params.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return GPET_OK;
}

int gpet_surrogate_set_params(gpet_surrogate* s, const float* in, int64_t n)
{
    if (!s || !in || n != s->nparam) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    SCK(cudaMemcpy(s->params.p, in, (size_t)n * 4, cudaMemcpyHostToDevice));
    int rc = refresh_weights(s);
    if (rc) return rc;
    SCK(cudaStreamSynchronize(s->stream));
    return GPET_OK;
}

int gpet_surrogate_get_cell_weights(gpet_surrogate* s, float* out, int64_t n)
{
    if (!s || !out || n != 2048) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    SCK(cudaMemcpy(out, s->corr.p, 2048 * 4, cudaMemcpyDeviceToHost));
    return GPET_OK;
}

int gpet_surrogate_set_cell_weights(gpet_surrogate* s, const float* in, int64_t n)
{
    if (!s || !in || n != 2048) return GPET_ERR_ARG;
    for (int64_t i = 0; i < n; ++i)
        if (!(in[i] >= 0.0f) || !std::isfinite(in[i])) return sfail(s, GPET_ERR_ARG, "cell weights must be finite, >= 0");
    SCK(cudaSetDevice(s->device));
    SCK(cudaMemcpy(s->corr.p, in, 2048 * 4, cudaMemcpyHostToDevice));
    return GPET_OK;
}

int gpet_surrogate_set_domain(gpet_surrogate* s, float e_lo, float e_hi, float margin, const uint8_t* panel_ok,
                              int32_t npanels)
{
    if (!s || !(e_lo >= 0.0f) || !(e_hi >= e_lo) || !(margin >= 0.0f)) return GPET_ERR_ARG;
    if (panel_ok && npanels != s->geom.npanels) return sfail(s, GPET_ERR_ARG, "one flag per panel");
    SCK(cudaSetDevice(s->device));
    s->e_lo = e_lo;
    s->e_hi = e_hi;
    s->margin = margin;
    if (panel_ok) {
        s->panel_ok.assign(panel_ok, panel_ok + npanels);
        SCK(cudaMemcpy(s->panel_ok_d.p, s->panel_ok.data(), s->panel_ok.size(), cudaMemcpyHostToDevice));
    }
    return GPET_OK;
}

int gpet_surrogate_grad(gpet_surrogate* s, const gpet_entry* rec, int64_t n, float* loss, float* grad)
{
    if (!s || !rec || n < 1 || !loss) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    int rc = ensure_batch(s, n);
    if (rc) return rc;
    SCK(cudaMemcpyAsync(s->rec.p, rec, (size_t)n * sizeof(EntryRec), cudaMemcpyHostToDevice, s->stream));
    rc = loss_and_grad(s, n, loss);
    if (rc) return rc;
    if (grad) SCK(cudaMemcpy(grad, s->grads.p, (size_t)s->nparam * 4, cudaMemcpyDeviceToHost));
    return GPET_OK;
}

int gpet_surrogate_forward(gpet_surrogate* s, const gpet_entry* rec, int64_t n, float* out208)
{
    if (!s || !rec || n < 1 || !out208) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    float loss = 0.0f;
    int rc = gpet_surrogate_grad(s, rec, n, &loss, nullptr);
    if (rc) return rc;
    SCK(cudaMemcpy(out208, s->out.p, (size_t)n * sg::kOut * 4, cudaMemcpyDeviceToHost));
    return GPET_OK;
}

int gpet_surrogate_train(gpet_surrogate* s, const gpet_entry* rec, int64_t n, int32_t epochs, int32_t batch,
                         float lr, uint64_t seed, float* epoch_loss)
{
    if (!s || !rec || n < 1 || epochs < 1 || batch < 128 || !(lr > 0.0f)) return GPET_ERR_ARG;
    if (n > (int64_t)UINT32_MAX) return sfail(s, GPET_ERR_ARG, "at most 2^32 - 1 training records");
    SCK(cudaSetDevice(s->device));
    const int64_t B = std::min<int64_t>(batch, n);
    int rc = ensure_batch(s, B);
    if (rc) return rc;
    // the training set goes to the device once; each epoch uploads a new
    // shuffled visiting order and the batches are gathered there
    SCK(s->all.ensure((size_t)n * sizeof(EntryRec)));
    SCK(s->perm.ensure((size_t)n * 4));
    SCK(s->epoch_loss.ensure(4));
    SCK(cudaMemcpyAsync(s->all.p, rec, (size_t)n * sizeof(EntryRec), cudaMemcpyHostToDevice, s->stream));
    std::vector<uint32_t> order((size_t)n);
    for (int64_t i = 0; i < n; ++i) order[(size_t)i] = (uint32_t)i;
    uint64_t st = seed;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    // learning rate: cosine from lr down to lr / 50 over the run's steps
    const int64_t steps = (int64_t)epochs * (n / B);
    int64_t step = 0;
    const unsigned gb = (unsigned)std::min<int64_t>((B + 255) / 256, 152 * 8);
    for (int ep = 0; ep < epochs; ++ep) {
        for (int64_t i = n - 1; i > 0; --i) std::swap(order[(size_t)i], order[(size_t)(splitmix(st) % (uint64_t)(i + 1))]);
        // the previous epoch's batches read the order buffer until they are done
        SCK(cudaStreamSynchronize(s->stream));
        SCK(cudaMemcpyAsync(s->perm.p, order.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
        SCK(cudaMemsetAsync(s->epoch_loss.p, 0, 4, s->stream));
        int64_t nb = 0;
        for (int64_t b0 = 0; b0 + B <= n; b0 += B) {
            k_gather_records<<<gb, 256, 0, s->stream>>>(s->all.as<EntryRec>(), s->perm.as<uint32_t>() + b0, B,
                                                       s->rec.as<EntryRec>());
            SCK(cudaGetLastError());
            rc = loss_and_grad(s, B, nullptr, s->epoch_loss.as<float>());
            if (rc) return rc;
            s->adam_t++;
            const float c1 = 1.0f / (1.0f - std::pow(b1, (float)s->adam_t));
            const float c2 = 1.0f / (1.0f - std::pow(b2, (float)s->adam_t));
            const double frac = steps > 1 ? (double)step / (double)(steps - 1) : 1.0;
            const float lr_t = (float)(lr * (0.02 + 0.49 * (1.0 + std::cos(3.14159265358979 * frac))));
            step++;
            k_adam<<<152 * 4, 256, 0, s->stream>>>(s->params.as<float>(), s->grads.as<float>(), s->adam_m.as<float>(),
                                                   s->adam_v.as<float>(), s->nparam, lr_t, b1, b2, eps, c1, c2);
            SCK(cudaGetLastError());
            rc = refresh_weights(s);
            if (rc) return rc;
            nb++;
        }
        float lsum = 0.0f;
        int herr = 0;
        SCK(cudaMemcpyAsync(&lsum, s->epoch_loss.p, 4, cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaMemcpyAsync(&herr, s->errflag.p, 4, cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaStreamSynchronize(s->stream));
        if (herr) return sfail(s, GPET_ERR_CUDA, "a tensor-core wait gave up");
        if (epoch_loss) epoch_loss[ep] = nb ? lsum / (float)nb : 0.0f;
    }
    SCK(cudaStreamSynchronize(s->stream));
    return GPET_OK;
}

int gpet_surrogate_calibrate(gpet_surrogate* s, const gpet_entry* rec, int64_t n, int32_t iters, float* max_adjust)
{
    using namespace sg;
    if (!s || !rec || n < 1 || iters < 1) return GPET_ERR_ARG;
    SCK(cudaSetDevice(s->device));
    const SurrogateDev sd = make_view(s);
    const int ncry = s->geom.crystalN;
    // the records of the surrogate's domain (the test of k_route) and their
    // observed (energy class, crystal) and energy-bin counts, the bin as in
    // training (0: no pulse)
    // joint head: (class, crystal) cells then the bins; factorised head: the
    // 2 x 32 x 32 (class, row, column) cells then the bins
    const int ebin0 = sd.fact ? 2048 : 2 * kCry;
    const int kAcc = ebin0 + kBins;
    const EntryRec* r = reinterpret_cast<const EntryRec*>(rec);
    std::vector<EntryRec> dom;
    std::vector<double> obs(kAcc, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        const EntryRec& e = r[i];
        const bool in = e.E >= s->e_lo && e.E <= s->e_hi && std::fabs(e.y) <= sd.half_y - s->margin &&
                        std::fabs(e.z) <= sd.half_z - s->margin && e.panel >= 0 && e.panel < s->geom.npanels &&
                        (s->panel_ok.empty() || s->panel_ok[(size_t)e.panel]);
        if (!in) continue;
        dom.push_back(e);
        int b = 0;
        if (e.crystal >= 0 && e.Edep > 0.0f) {
            b = (int)(e.Edep / e.E * (float)kBins);
            b = b < 1 ? 1 : (b > kBins - 1 ? kBins - 1 : b);
            const int set = b >= kClassBin ? 1 : 0;
            if (e.crystal < ncry) {
                if (sd.fact)
                    obs[(size_t)(set * 1024 + (e.crystal % sd.crystalNy) * 32 + e.crystal / sd.crystalNy)] += 1.0;
                else
                    obs[(size_t)(set * kCry + e.crystal)] += 1.0;
            }
        }
        obs[(size_t)(ebin0 + b)] += 1.0;
    }
    const int64_t m = (int64_t)dom.size();
    if (m == 0) return sfail(s, GPET_ERR_ARG, "no record in the surrogate's domain");
    const int64_t B = std::min<int64_t>(m, 1 << 16);
    int rc = ensure_batch(s, B);
    if (rc) return rc;
    SCK(s->all.ensure((size_t)m * sizeof(EntryRec)));
    SCK(s->calib.ensure(kAcc * sizeof(double)));
    SCK(cudaMemcpyAsync(s->all.p, dom.data(), (size_t)m * sizeof(EntryRec), cudaMemcpyHostToDevice, s->stream));
    const int smem = (int)(kSmemA + kSmemB);
    SCK(cudaFuncSetAttribute(k_mlp_fwd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    float last = 0.0f;
    for (int it = 0; it < iters; ++it) {
        SCK(cudaMemsetAsync(s->calib.p, 0, kAcc * sizeof(double), s->stream));
        for (int64_t b0 = 0; b0 < m; b0 += B) {
            const int64_t nb = std::min<int64_t>(B, m - b0);
            SCK(cudaMemcpyAsync(s->rec.p, s->all.as<EntryRec>() + b0, (size_t)nb * sizeof(EntryRec),
                                cudaMemcpyDeviceToDevice, s->stream));
            const unsigned g1 = (unsigned)std::min<int64_t>((nb + 255) / 256, 152 * 8);
            k_entry_features<<<g1, 256, 0, s->stream>>>(s->rec.as<EntryRec>(), nb, sd, s->params.as<float>(),
                                                        s->X.as<__nv_bfloat16>(), s->cry.as<int32_t>(),
                                                        s->dep.as<float>(), s->bin.as<int32_t>(),
                                                        s->pan.as<int32_t>());
            FwdTrain tr{s->X.as<__nv_bfloat16>(), nb, s->Z.as<float>(), s->H.as<__nv_bfloat16>(), s->out.as<float>()};
            FwdInfer in{};
            k_mlp_fwd<true><<<grid_cap(nb, 128, 152), kFwdThreads, smem, s->stream>>>(sd, tr, in,
                                                                                     s->errflag.as<int>());
            if (sd.fact)
                k_calib_accum_grid<<<(unsigned)std::min<int64_t>((nb + 7) / 8, 152 * 8), 256, 0, s->stream>>>(
                    s->out.as<float>(), nb, sd.crystalNy, sd.crystalNz, sd.corr, s->calib.as<double>());
            else
                k_calib_accum<<<(unsigned)std::min<int64_t>((nb + 7) / 8, 152 * 8), 256, 0, s->stream>>>(
                    s->out.as<float>(), nb, ncry, s->calib.as<double>());
            SCK(cudaGetLastError());
        }
        std::vector<double> expd(kAcc);
        std::vector<float> bias(kOut);
        int herr = 0;
        float* const pb = s->params.as<float>() + b_off(kLayers - 1);
        SCK(cudaMemcpyAsync(expd.data(), s->calib.p, expd.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaMemcpyAsync(bias.data(), pb, bias.size() * 4, cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaMemcpyAsync(&herr, s->errflag.p, 4, cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaStreamSynchronize(s->stream));
        if (herr) return sfail(s, GPET_ERR_CUDA, "a tensor-core wait gave up");
        // the crystal logits of each class (factorised head: the cell
        // weights) and the energy-bin logits move by log(observed / expected)
        last = 0.0f;
        auto ratio = [&](size_t j, float* d) {
            if (!(obs[j] > 0.0) || !(expd[j] > 0.0)) return false;
            *d = (float)std::log(obs[j] / expd[j]);
            last = std::max(last, std::fabs(*d));
            return true;
        };
        float d = 0.0f;
        if (sd.fact) {
            std::vector<float> w(2048);
            SCK(cudaMemcpyAsync(w.data(), s->corr.p, w.size() * 4, cudaMemcpyDeviceToHost, s->stream));
            SCK(cudaStreamSynchronize(s->stream));
            for (int set = 0; set < 2; ++set)
                for (int ky = 0; ky < sd.crystalNy; ++ky)
                    for (int kz = 0; kz < sd.crystalNz; ++kz) {
                        const size_t j = (size_t)(set * 1024 + ky * 32 + kz);
                        if (ratio(j, &d)) w[j] *= std::exp(d);
                    }
            SCK(cudaMemcpyAsync(s->corr.p, w.data(), w.size() * 4, cudaMemcpyHostToDevice, s->stream));
        } else {
            for (int set = 0; set < 2; ++set)
                for (int k = 0; k < ncry; ++k)
                    if (ratio((size_t)(set * kCry + k), &d)) bias[(size_t)(set * kCry + k)] += d;
        }
        for (int b = 0; b < kBins; ++b)
            if (ratio((size_t)(ebin0 + b), &d)) bias[(size_t)(kColE + b)] += d;
        SCK(cudaMemcpyAsync(pb, bias.data(), bias.size() * 4, cudaMemcpyHostToDevice, s->stream));
        rc = refresh_weights(s);
        if (rc) return rc;
        SCK(cudaStreamSynchronize(s->stream));
    }
    if (max_adjust) *max_adjust = last;
    return GPET_OK;
}

}  // extern "C"
