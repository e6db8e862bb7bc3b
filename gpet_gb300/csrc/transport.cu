// transport.cu - source, positron range, annihilation, phantom and detector
// transport kernels (the work of setPosition/setPositionForPhoton, photon and
// photonde in gPET_kernals.cu:256-1233), for sm_103a.
//
// Layout: k_source runs one thread per decay and writes the emitted pairs to
// an L2-resident structure-of-arrays buffer; k_phantom keeps persistent warps
// whose lanes refill themselves with the next photon as soon as their photon
// leaves the phantom, and compacts photons that reach a panel (warp ballot,
// one atomic per warp) into the detector queue; k_detector runs one thread per
// queued photon through the panel, applies the per-photon adder and readout,
// and appends pulses and hits (one atomic per warp).
#include <cstddef>

#include "kernels.h"

namespace gpet {

// the simulation's descriptor (its first `bytes` bytes) and panels into
// shared memory
__device__ __forceinline__ void load_sim(const SimDesc* __restrict__ g, SimDesc& s, float* sP,
                                         size_t bytes = sizeof(SimDesc))
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(g);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s);
    for (int i = threadIdx.x; i < (int)(bytes / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    int np = s.npanels * kPanelStride;
    for (int i = threadIdx.x; i < np; i += blockDim.x) sP[i] = __ldg(s.panels + i);
    __syncthreads();
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// segment table of a wave, staged in shared memory
struct SegSmem {
    int64_t g0[kMaxSeg + 1];
    int64_t d0[kMaxSeg];
    int32_t sim[kMaxSeg];
    int32_t nseg;
};

__device__ __forceinline__ void load_segs(const Wave& w, SegSmem& sg)
{
    for (int i = threadIdx.x; i <= w.nseg; i += blockDim.x) sg.g0[i] = w.g0[i];
    for (int i = threadIdx.x; i < w.nseg; i += blockDim.x) {
        sg.d0[i] = w.d0[i];
        sg.sim[i] = w.sim[i];
    }
    if (threadIdx.x == 0) sg.nseg = w.nseg;
}

// segment holding global decay index g (g0 ascending)
__device__ __forceinline__ int seg_of(const SegSmem& sg, int64_t g)
{
    int lo = 0, hi = sg.nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (sg.g0[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// source stage of one decay (setPosition gPET_kernals.cu:483-561 for a source
// in the H3 form: the decay's source is fixed by its index, its time is a
// truncated exponential on [0, dt)); PSF records (setPositionForPhoton
// :563-604, with the second photon's time set) when npsf > 0.
// Returns how many photons of the pair exist (0, 1 or 2). walk: the positron
// range needs the voxel walk, which starts at the pair's position with
// displacement wd[0..2] of length wd[3], density-weighted length wd[5]
// already covered and about wd[4] steps to go (the pair's position is then
// the walk's start, and k_walk moves it).
__device__ int sample_decay(const SimDesc& S, int64_t d, Photon ph[2], bool& walk, float wd[6])
{
    Stream st;
    st_init(st, S.key0, S.key1, kTagDecay, (uint64_t)d);
    walk = false;
    if (S.npsf > 0) {
        const double* r = S.psf + 8 * d;
        if (S.psf_ptype == 1) {
            ph[0].x[0] = (float)r[0]; ph[0].x[1] = (float)r[1]; ph[0].x[2] = (float)r[2];
            ph[0].u[0] = (float)r[4]; ph[0].u[1] = (float)r[5]; ph[0].u[2] = (float)r[6];
            ph[0].E = (float)r[7]; ph[0].t = r[3]; ph[0].tf = 0.0f; ph[0].nscat = 0;
            return (r[3] > 0.0 && ph[0].E >= 0.0f) ? 1 : 0;
        }
        float pos[3] = {(float)r[0], (float)r[1], (float)r[2]};
        float dir[3] = {(float)r[4], (float)r[5], (float)r[6]};
        float spare = 0.0f;
        if (S.useprange) {
            wd[3] = prange_draw((float)r[7], dir, st, wd, &spare);
            walk = !prange_uniform(S, pos, wd, wd[3], wd[4], wd[5]);
        }
        make_pair(S, st, pos, r[3], ph, S.useprange ? &spare : nullptr);
        return 2;
    }
    int si = 0;
    while (si < S.nsrc - 1 && d >= S.src_end[si]) si++;
    double ud = st_ud(st);
    const double cf = S.src_cfac[si];
    const double xl = -ud * cf;
    // t = tstart - lifetime log(1 - u (1 - exp(-window / lifetime))), in us
    const double L = cf <= 0.015625 ? dm_log1p_small(xl) : dm_log(1.0 + xl);
    double t_us = dm_fmad(S.src_ntau_us[si], L, S.tstart_us);
    float br = st_u(st);
    if (!(br < S.iso_ratio[si])) return 0;
    float pos[3];
    shape_position(S, si, st, pos);
    float spare = 0.0f;
    if (S.useprange) {
        float ek = sample_ek(S.iso_coef[si], st);
        wd[3] = prange_draw(ek, nullptr, st, wd, &spare);
        walk = !prange_uniform(S, pos, wd, wd[3], wd[4], wd[5]);
    }
    make_pair(S, st, pos, t_us, ph, S.useprange ? &spare : nullptr);
    return 2;
}

// walk list of a positron walk of about `est` voxel steps
__device__ __forceinline__ int walk_list(float est)
{
    return est < 4.0f ? 0 : (est < 8.0f ? 1 : (est < 16.0f ? 2 : 3));
}

// source stage: one thread per decay, the emitted pair (or PSF photon) goes
// to a structure-of-arrays buffer. kMulti: the decays of a wave belong to
// several simulations and each thread reads its own simulation's descriptor;
// otherwise the one descriptor is staged in shared memory. Decays whose
// positron range needs the voxel walk are appended to one of the wave's
// kWalkLists walk lists by their estimated number of steps (one atomic per
// warp and list), and their position is written by k_walk.
template <bool kMulti>
__global__ void __launch_bounds__(256, 6) k_source(const Wave* waves, int wi, PairBuf pb, Counters* cnt)
{
    const Wave w = waves[wi];
    __shared__ SimDesc sS;
    __shared__ SegSmem sg;
    extern __shared__ float sP[];
    if (!kMulti) load_sim(w.sims, sS, sP);
    load_segs(w, sg);
    __syncthreads();
    const unsigned lt = lanemask_lt();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    SimTally pairs;
    // every lane of a warp runs the same iterations (base is block-uniform)
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < w.n; base += stride) {
        const int64_t j = base + threadIdx.x;
        int nph = 0;
        int sim = 0;
        bool walk = false;
        float wd[6];
        Photon ph[2];
        if (j < w.n) {
            const int sgi = seg_of(sg, j);
            sim = sg.sim[sgi];
            const int64_t d = sg.d0[sgi] + (j - sg.g0[sgi]);
            const SimDesc& S = kMulti ? w.sims[sim] : sS;
            nph = sample_decay(S, d, ph, walk, wd);
            pb.nph[j] = (uint8_t)nph;
            if (nph > 0) {
                if (!walk) {
                    pb.f[0 * pb.cap + j] = ph[0].x[0];
                    pb.f[1 * pb.cap + j] = ph[0].x[1];
                    pb.f[2 * pb.cap + j] = ph[0].x[2];
                }
                pb.f[3 * pb.cap + j] = ph[0].u[0];
                pb.f[4 * pb.cap + j] = ph[0].u[1];
                pb.f[5 * pb.cap + j] = ph[0].u[2];
                pb.f[9 * pb.cap + j] = ph[0].E;
                pb.t[j] = ph[0].t;
            }
            if (nph > 1) {
                pb.f[6 * pb.cap + j] = ph[1].u[0];
                pb.f[7 * pb.cap + j] = ph[1].u[1];
                pb.f[8 * pb.cap + j] = ph[1].u[2];
                pb.f[10 * pb.cap + j] = ph[1].E;
            }
            pairs.add(cnt, CF(pairs), sim, nph == 2 ? 1u : 0u);
        }
        if (__any_sync(0xffffffffu, walk)) {
            // lanes of one list take consecutive entries (one atomic per list)
            const int wl = walk ? walk_list(wd[4]) : -1;
            const unsigned grp = __match_any_sync(0xffffffffu, wl);
            if (walk) {
                const int leader = __ffs(grp) - 1;
                unsigned long long base_k = 0;
                if (lane == leader) base_k = atomicAdd(w.walkn + wl, (unsigned long long)__popc(grp));
                base_k = __shfl_sync(grp, base_k, leader);
                const unsigned long long k = base_k + __popc(grp & lt);
                float* wf = pb.wf + (size_t)wl * kWalkFields * pb.cap;
                wf[0 * pb.cap + k] = ph[0].x[0];
                wf[1 * pb.cap + k] = ph[0].x[1];
                wf[2 * pb.cap + k] = ph[0].x[2];
                wf[3 * pb.cap + k] = wd[0];
                wf[4 * pb.cap + k] = wd[1];
                wf[5 * pb.cap + k] = wd[2];
                wf[6 * pb.cap + k] = wd[3];
                wf[7 * pb.cap + k] = wd[5];
                pb.wj[(size_t)wl * pb.cap + k] = (int32_t)j;
            }
        }
    }
    pairs.flush(cnt, CF(pairs));
}

// the positron-range walks k_source left (prange_walk_*), list by list: a
// lane walks one positron to its end; the lists hold walks of similar
// estimated length, so the lanes of a warp finish at about the same step
// (a refill as soon as a lane's walk ends put the refill and the step on
// separate paths of the warp at nearly every step). The end point is the
// pair's position in the pair buffer. At most one entry per decay of the
// wave in each list, so no list overflows.
template <bool kMulti>
__global__ void __launch_bounds__(256) k_walk(const Wave* waves, int wi, PairBuf pb)
{
    const Wave w = waves[wi];
    __shared__ __align__(16) uint32_t sSw[kSimTransportBytes / 4];
    SimDesc& sS = *reinterpret_cast<SimDesc*>(sSw);
    __shared__ SegSmem sg;
    if (kMulti) {
        load_segs(w, sg);
    } else {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(w.sims);
        for (int i = threadIdx.x; i < (int)(kSimTransportBytes / 4); i += blockDim.x) sSw[i] = src[i];
    }
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int b = 0; b < kWalkLists; ++b) {
        const int64_t n = (int64_t)w.walkn[b];
        const float* wf = pb.wf + (size_t)b * kWalkFields * pb.cap;
        const int32_t* wj = pb.wj + (size_t)b * pb.cap;
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
            const int32_t j = wj[k];
            const float x[3] = {wf[0 * pb.cap + k], wf[1 * pb.cap + k], wf[2 * pb.cap + k]};
            const float d[3] = {wf[3 * pb.cap + k], wf[4 * pb.cap + k], wf[5 * pb.cap + k]};
            const float r = wf[6 * pb.cap + k], s0 = wf[7 * pb.cap + k];
            const SimDesc* S = kMulti ? w.sims + sg.sim[seg_of(sg, j)] : &sS;
            PWalk pw;
            if (prange_walk_init(*S, pw, x, d, r, s0))
                while (prange_walk_step(*S, pw)) {
                }
            pb.f[0 * pb.cap + j] = pw.x[0];
            pb.f[1 * pb.cap + j] = pw.x[1];
            pb.f[2 * pb.cap + j] = pw.x[2];
        }
    }
}

// a photon that has left the phantom (or stopped), waiting for the panel search
// (always escaped: status 1; the emission time stays in the pair buffer and
// is read in the drain, only for the photons that need it; the decay index
// and simulation follow from the photon index through the wave's segments)
struct FinRec {
    float x, y, z, ux, uy, uz, E;
    int32_t nscat;
    int32_t p;        // photon index within the wave
    float tf;
};
static_assert(sizeof(FinRec) == 40, "staged record");

constexpr int kPhWarps = 8;      // warps per k_phantom block (256 threads)
constexpr uint32_t kClaim = 128; // photons a k_phantom warp claims at a time
constexpr int kFinCap = 64;      // finished photons staged per warp

// phantom stage: persistent warps; a lane whose photon has left the phantom
// (or was absorbed) takes the next photon from a shared counter at once, so
// the lanes of a warp stay busy while histories differ in length. Finished
// photons are staged in shared memory and taken through the panel search 32
// at a time, one per lane. Photon p of the wave is photon (p & 1) of the
// wave's decay p >> 1. kMulti as for k_source.
template <bool kMulti>
__global__ void __launch_bounds__(256, 5) k_phantom(const Wave* waves, int wi, PairBuf pb, QueueDev q, Counters* cnt,
                                                    int period)
{
    const Wave w = waves[wi];
    unsigned long long* const work = w.work;
    ExitRec* const exits = w.exits;
    // the descriptor's transport part only (the sources are k_source's)
    __shared__ __align__(16) uint32_t sSw[kSimTransportBytes / 4];
    SimDesc& sS = *reinterpret_cast<SimDesc*>(sSw);
    __shared__ SegSmem sg;
    __shared__ FinRec fbuf[kPhWarps][kFinCap];
    extern __shared__ float sP[];
    if (!kMulti) load_sim(w.sims, sS, sP, kSimTransportBytes);
    load_segs(w, sg);
    __syncthreads();
    const unsigned lt = lanemask_lt();
    const int lane = threadIdx.x & 31;
    FinRec* fb = fbuf[threadIdx.x >> 5];
    const int64_t nphot = 2 * w.n;
    int fcount = 0;   // staged photons of this warp (warp-uniform)

    // panel search + queue append for the staged entries [0, k), one per lane
    // (escaped photons that may reach a panel)
    auto drain = [&](int k) {
        const bool has = lane < k;
        FinRec r;
        int rsim = 0;
        int64_t rd = 0;
        if (has) {
            r = fb[lane];
            const int64_t j = r.p >> 1;
            const int sgi = seg_of(sg, j);
            rsim = kMulti ? sg.sim[sgi] : 0;
            rd = sg.d0[sgi] + (j - sg.g0[sgi]);
        }
        Photon ph;
        Local L;
        bool entered = false;
        if (has) {
            ph.x[0] = r.x; ph.x[1] = r.y; ph.x[2] = r.z;
            ph.u[0] = r.ux; ph.u[1] = r.uy; ph.u[2] = r.uz;
            ph.E = r.E; ph.t = 0.0; ph.tf = r.tf; ph.nscat = r.nscat;   // L.t: flight time alone
            if (kMulti) {
                const SimDesc& S = w.sims[rsim];
                entered = enter_panel(S.panels, S.npanels, ph, L);
            } else {
                entered = enter_panel(sP, sS.npanels, ph, L);
            }
        }
        // the emission time, loaded by all lanes that need it at once
        const double te = (entered || (has && exits)) ? pb.t[r.p >> 1] : 0.0;
        if (entered) L.t = te + L.t;
        const unsigned m = __ballot_sync(0xffffffffu, entered);
        if (m) {
            unsigned long long b = 0;
            const int leader = __ffs(m) - 1;
            if (lane == leader) b = atomicAdd(q.count, (unsigned long long)__popc(m));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (entered) {
                const unsigned long long jq = b + __popc(m & lt);
                if (jq < (unsigned long long)q.cap) {
                    const int64_t d = rd;
                    q.f[0 * q.cap + jq] = L.x[0];
                    q.f[1 * q.cap + jq] = L.x[1];
                    q.f[2 * q.cap + jq] = L.x[2];
                    q.f[3 * q.cap + jq] = L.u[0];
                    q.f[4 * q.cap + jq] = L.u[1];
                    q.f[5 * q.cap + jq] = L.u[2];
                    q.f[6 * q.cap + jq] = L.E;
                    q.t[jq] = L.t;
                    q.i[0 * q.cap + jq] = L.panel;
                    q.i[1 * q.cap + jq] = (int32_t)(2 * d + (r.p & 1));
                    q.i[2 * q.cap + jq] = (int32_t)d;
                    q.i[3 * q.cap + jq] = r.nscat;
                    q.i[4 * q.cap + jq] = rsim;
                } else {
                    entered = false;
                    atomicAdd(&cnt->queue_drop, 1ull);
                }
            }
        }
        add_by_sim(cnt, rsim, CF(entered), entered ? 1u : 0u);
        if (has && exits) {
            ExitRec e;
            e.x = r.x; e.y = r.y; e.z = r.z; e.ux = r.ux; e.uy = r.uy; e.uz = r.uz;
            e.E = r.E; e.nscat = r.nscat; e.t = te + (double)r.tf;
            e.status = 1;
            e.panel = entered ? L.panel : -1;
            exits[r.p] = e;
        }
        __syncwarp();
    };

    bool active = false, exhausted = false;
    int32_t p = 0;   // photon index within the wave (< 2^25)
    int64_t d = 0;
    int sim = 0;
    int steps = 0;
    SimTally t_steps;
    Photon ph;
    // the photon's stream (tag kTagPhantom + (p & 1), id d, the simulation's
    // key), seeded when the lane takes the photon
    uint32_t rst[4] = {0u, 0u, 0u, 0u};
    auto unif = [&]() -> float { return dm_u01(xo_next(rst)); };
    // The warp claims photons kClaim at a time, one block ahead of the lanes
    // that take them, and has the next block's pair-buffer lines fetched
    // into L2 when it claims it: a lane's refill then reads L2 instead of
    // waiting for DRAM while its warp's other lanes wait for it.
    // [cb, ce): the block lanes take photons from; nb: the next block.
    auto claim = [&]() -> uint32_t {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(work, (unsigned long long)kClaim);
        const uint32_t b = (uint32_t)__shfl_sync(0xffffffffu, t, 0);
        if (b < (uint32_t)nphot) {
            // every 128-byte line of decays [b/2, b/2 + kClaim/2) in the 11
            // float arrays, the emission times and the photon counts: the
            // lanes take the (array, line) pairs in turn; the range's last
            // element is prefetched too (the range need not start on a line)
            const int64_t j0 = b >> 1;
            const int64_t nd = min((int64_t)(kClaim / 2), w.n - j0);
            constexpr int kFl = kClaim / 64 + 1, kTl = kClaim / 32 + 1;   // lines per float / time array
            for (int q = lane; q < 11 * kFl + kTl + 1; q += 32) {
                const void* ptr;
                if (q < 11 * kFl) {
                    const int64_t o = min((int64_t)(q % kFl) * 32, nd - 1);
                    ptr = pb.f + (q / kFl) * pb.cap + j0 + o;
                } else if (q < 11 * kFl + kTl) {
                    ptr = pb.t + j0 + min((int64_t)(q - 11 * kFl) * 16, nd - 1);
                } else {
                    ptr = pb.nph + j0;
                }
                asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
            }
        }
        return b;
    };
    uint32_t cb = claim();
    uint32_t ce = cb + kClaim;
    uint32_t nb = claim();
    for (;;) {
        // refill idle lanes from the claimed blocks
        const bool need = !active && !exhausted;
        const unsigned mneed = __ballot_sync(0xffffffffu, need);
        if (mneed) {
            const uint32_t k = __popc(mneed), r = __popc(mneed & lt), avail = ce - cb;
            const uint32_t pw = r < avail ? cb + r : nb + (r - avail);
            if (k >= avail) {   // into the next block (k <= 32 <= kClaim): claim the one after it
                cb = nb + (k - avail);
                ce = nb + kClaim;
                nb = claim();
            } else {
                cb += k;
            }
            if (need) {
                if (pw >= (uint32_t)nphot) {
                    exhausted = true;
                } else {
                    p = (int32_t)pw;
                    const int64_t j = p >> 1;
                    const int k = (int)(p & 1);
                    const int sgi = seg_of(sg, j);
                    sim = kMulti ? sg.sim[sgi] : 0;
                    d = sg.d0[sgi] + (j - sg.g0[sgi]);
                    const int nph = pb.nph[j];
                    if (k < nph) {
                        ph.x[0] = pb.f[0 * pb.cap + j];
                        ph.x[1] = pb.f[1 * pb.cap + j];
                        ph.x[2] = pb.f[2 * pb.cap + j];
                        ph.u[0] = pb.f[(3 + 3 * k) * pb.cap + j];
                        ph.u[1] = pb.f[(4 + 3 * k) * pb.cap + j];
                        ph.u[2] = pb.f[(5 + 3 * k) * pb.cap + j];
                        ph.E = pb.f[(9 + k) * pb.cap + j];
                        ph.t = 0.0;   // the emission time stays in the pair buffer (pb.t[p >> 1])
                        ph.tf = 0.0f;
                        ph.nscat = 0;
                        {
                            const SimDesc& S = kMulti ? w.sims[sim] : sS;
                            st_seed(rst, S.key0, S.key1, kTagPhantom + (uint32_t)(p & 1), (uint32_t)d,
                                    (uint32_t)((uint64_t)d >> 32));
                        }
                        steps = 0;
                        active = true;
                        if (w.source) {
                            SrcRec r;
                            r.x = ph.x[0]; r.y = ph.x[1]; r.z = ph.x[2];
                            r.ux = ph.u[0]; r.uy = ph.u[1]; r.uz = ph.u[2];
                            r.E = ph.E; r.eventid = (int32_t)d; r.t = pb.t[j];
                            w.source[p] = r;
                        }
                    } else {
                        if (exits) {
                            ExitRec e;
                            e.x = e.y = e.z = e.ux = e.uy = e.uz = e.E = 0.0f; e.nscat = 0; e.t = 0.0;
                            e.status = 2; e.panel = -1;
                            exits[p] = e;
                        }
                        if (w.source) {
                            SrcRec r;
                            r.x = r.y = r.z = r.ux = r.uy = r.uz = r.E = 0.0f; r.eventid = 0; r.t = 0.0;
                            w.source[p] = r;
                        }
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, !active && exhausted)) break;
        // one Woodcock step (photon(), gPET_kernals.cu:274-338)
        int status = -1;   // -1 continue, 0 absorbed, 1 escaped, 3 step cap
        if (active) {
            const SimDesc& S = kMulti ? w.sims[sim] : sS;
            steps++;
            float lammin = wck_at(S.wck_ph, S.wck_e0, S.wck_ide, ph.E);
            float s = -lammin * dm_logf(unif());
            ph.x[0] = dm_fma(s, ph.u[0], ph.x[0]);
            ph.x[1] = dm_fma(s, ph.u[1], ph.x[1]);
            ph.x[2] = dm_fma(s, ph.u[2], ph.x[2]);
            ph.tf = dm_fma(s, DM_INV_SPEED, ph.tf);
            int ix, iy, iz;
            if (!abs_vox(S, ph.x[0], ph.x[1], ph.x[2], ix, iy, iz)) {
                status = 1;
            } else {
                uint2 vv = voxel(S, ix, iy, iz);
                float voxden = __uint_as_float(vv.x);
                int m = (int)vv.y;
                float lamden = lammin * voxden;
                float4 xs = xs_at(S, m, ph.E);
                float prob = dm_fma(-lamden, xs.x, 1.0f);
                float rn = unif();
                if (rn < prob) {
                } else {
                    prob = dm_fma(lamden, xs.y, prob);
                    if (rn < prob) {
                        float efrac, cost;
                        compton_surface_u(S, ph.E, m, unif, efrac, cost);
                        float phi = unif();
                        ph.E *= efrac;
                        ph.nscat++;
                        if (ph.E < S.eabsph) status = 1;
                        else rotate(ph.u[0], ph.u[1], ph.u[2], cost, phi);
                    } else {
                        prob = dm_fma(lamden, xs.z, prob);
                        if (rn < prob) {
                            float cost = rayleigh_surface_u(S, ph.E, m, unif);
                            float phi = unif();
                            rotate(ph.u[0], ph.u[1], ph.u[2], cost, phi);
                            ph.nscat++;
                        } else {
                            status = 0;
                        }
                    }
                }
            }
            if (status < 0 && steps >= kMaxSteps) status = 3;
        }
        // a finished photon that may reach a panel is staged for the panel
        // search, which runs once 32 are waiting (full warps); the others
        // (absorbed, step cap, or no panel within reach) are settled here
        const bool fin = status >= 0;
        bool search = false;
        if (fin) {
            const SimDesc& S = kMulti ? w.sims[sim] : sS;
            search = status == 1 && may_reach_panels(S, ph);
            t_steps.add(cnt, CF(ph_steps), sim, (unsigned)steps);
            if (status == 3) atomicAdd(&cnt[sim].stepcap, 1ull);
            if (!search) {
                if (exits) {
                    ExitRec e;
                    e.x = ph.x[0]; e.y = ph.x[1]; e.z = ph.x[2];
                    e.ux = ph.u[0]; e.uy = ph.u[1]; e.uz = ph.u[2];
                    e.E = ph.E; e.nscat = ph.nscat; e.t = pb.t[p >> 1] + (double)ph.tf;
                    e.status = status;
                    e.panel = -1;
                    exits[p] = e;
                }
                active = false;
            }
        }
        const unsigned mf = __ballot_sync(0xffffffffu, search);
        if (mf) {
            if (search) {
                FinRec r;
                r.x = ph.x[0]; r.y = ph.x[1]; r.z = ph.x[2];
                r.ux = ph.u[0]; r.uy = ph.u[1]; r.uz = ph.u[2];
                r.E = ph.E; r.nscat = ph.nscat; r.p = p; r.tf = ph.tf;
                fb[fcount + __popc(mf & lt)] = r;
                active = false;
            }
            fcount += __popc(mf);
            __syncwarp();
            // fcount <= 31 before staging, so <= 63 < kFinCap here, and the
            // rest after a drain of min(fcount, 32) is <= 31 again
            if (fcount >= period) {
                const int k = fcount < 32 ? fcount : 32;
                drain(k);
                const int rest = fcount - k;
                FinRec r;
                if (lane < rest) r = fb[k + lane];
                __syncwarp();
                if (lane < rest) fb[lane] = r;
                __syncwarp();
                fcount = rest;
            }
        }
    }
    if (fcount > 0) drain(fcount);
    t_steps.flush(cnt, CF(ph_steps));
}

// ------------------------------------------------------------- detector
// a deposit of one photon: all of them lie in the photon's panel, so module
// and crystal identify the crystal (the site number follows from them)
struct PEvent {
    int32_t modn, cryn;
    double t;
    float E, x, y, z;
};

// the pulse's site number after readout at the configured depth
// (setSitenum levels of gPET_kernals.cu:778-808: depth 3 and up keep the crystal)
__device__ __forceinline__ int32_t site_of(const SimDesc& S, int32_t pann, int32_t modn, int32_t cryn)
{
    const int depth = S.rdepth == 3 ? 3 : (S.rpolicy == 1 ? 2 : S.rdepth);
    if (depth == 0) return 0;
    if (depth == 1) return pann;
    if (depth == 2) return pann * S.moduleN + modn;
    return pann * S.moduleN * S.crystalN + modn * S.crystalN + cryn;
}

// adder, gPET_kernals.cu:737-755 (same crystal: same module and crystal)
__device__ __forceinline__ bool adder(PEvent* ev, int& n, const PEvent& e)
{
    for (int i = 0; i < n; ++i) {
        if (e.modn == ev[i].modn && e.cryn == ev[i].cryn) {
            float s = ev[i].E + e.E;
            ev[i].x = (ev[i].x * ev[i].E + e.x * e.E) / s;
            ev[i].y = (ev[i].y * ev[i].E + e.y * e.E) / s;
            ev[i].z = (ev[i].z * ev[i].E + e.z * e.E) / s;
            ev[i].E = ev[i].E + e.E;
            return true;
        }
    }
    if (n >= kMaxPulse) return false;
    ev[n++] = e;
    return true;
}

// readout, gPET_kernals.cu:756-813 (in place; depth 3 keeps the list)
__device__ __forceinline__ int readout(const SimDesc& S, PEvent* ev, int n)
{
    int depth = S.rdepth, policy = S.rpolicy;
    if (depth == 3) return n;
    if (policy == 1) depth = 2;
    // the site at this depth within the photon's panel: all one site at
    // depths 0 and 1, the module at 2, the crystal above
    auto key = [&](const PEvent& e) -> int32_t {
        return depth <= 1 ? 0 : (depth == 2 ? e.modn : e.modn * S.crystalN + e.cryn);
    };
    unsigned dead = 0;
    int k = 0;
    for (int i = 0; i < n; ++i) {
        if (dead & (1u << i)) continue;
        PEvent e0 = ev[i];
        for (int j = i + 1; j < n; ++j) {
            const PEvent e = ev[j];
            if (key(e) == key(e0)) {   // one photon: parn always equal
                if (policy == 1) {
                    float s = e0.E + e.E;
                    e0.x = (e0.x * e0.E + e.x * e.E) / s;
                    e0.y = (e0.y * e0.E + e.y * e.E) / s;
                    e0.z = (e0.z * e0.E + e.z * e.E) / s;
                    e0.E = e0.E + e.E;
                } else {
                    e0 = (e0.E > e.E) ? e0 : e;
                }
                dead |= 1u << j;
            }
        }
        ev[k++] = e0;
    }
    return k;
}

// Detector stage: persistent warps; a lane whose photon has finished takes
// the next queued photon at once (one atomic per warp), so the lanes stay busy
// while photons need different numbers of steps; pulses and hits of the
// photons that finished in an iteration are appended with one atomic per warp.
// kMulti as for k_source: the queue holds photons of several simulations.
template <bool kMulti>
__global__ void __launch_bounds__(256, 3) k_detector(const SimDesc* sims, QueueDev q, PulseDev P,
                                                  HitDev H, int rec_hits, Counters* cnt, EntryRec* entries)
{
    __shared__ __align__(16) uint32_t sSw[kSimTransportBytes / 4];
    SimDesc& sS = *reinterpret_cast<SimDesc*>(sSw);
    extern __shared__ float sP[];
    if (!kMulti) {
        load_sim(sims, sS, sP, kSimTransportBytes);
        __syncthreads();
    }
    unsigned long long nq = *q.count;
    if (nq > (unsigned long long)q.cap) nq = (unsigned long long)q.cap;
    const int64_t n = (int64_t)nq;
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    unsigned long long n_pdrop = 0, n_hdrop = 0;
    SimTally t_steps, t_cap, t_over, t_pulse, t_hit;
    // the lane's photon
    bool active = false, exhausted = false;
    int64_t j = 0;
    Local L;
    const float* Pn = nullptr;
    int32_t pann = 0;
    PEvent ev[kMaxPulse];
    int nev = 0, nh = 0, step = 0;
    int32_t parn = 0, eid = 0, scat = 0, sim = 0;
    bool overflow = false;
    unsigned nsteps = 0;
    EntryRec er;
    // the photon's stream (tag kTagDet + (parn & 1), id eid, the simulation's
    // key), seeded when the lane takes the photon
    uint32_t rst[4] = {0u, 0u, 0u, 0u};
    // a deposit goes to the hit list at once (at most kMaxHits per photon),
    // the lanes that record one at the same point sharing one atomic
    auto put_hit = [&](int32_t M_id, int32_t L_id, int32_t type, float Ed, double t) {
        if (nh >= kMaxHits) {
            overflow = true;
            return;
        }
        nh++;
        const unsigned act = __activemask();
        const int leader = __ffs(act) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(H.count, (unsigned long long)__popc(act));
        base = __shfl_sync(act, base, leader);
        const unsigned long long o = base + __popc(act & lt);
        if (o >= (unsigned long long)H.cap) {
            n_hdrop++;
            return;
        }
        H.id[5 * o + 0] = parn;
        H.id[5 * o + 1] = pann; H.id[5 * o + 2] = M_id; H.id[5 * o + 3] = L_id; H.id[5 * o + 4] = type;
        H.f[5 * o + 0] = Ed; H.f[5 * o + 1] = (float)t;
        H.f[5 * o + 2] = L.x[0]; H.f[5 * o + 3] = L.x[1]; H.f[5 * o + 4] = L.x[2];
        if (H.sim) H.sim[o] = sim;
    };
    auto unif = [&]() -> float { return dm_u01(xo_next(rst)); };
    for (;;) {
        // refill idle lanes
        const bool need = !active && !exhausted;
        const unsigned mneed = __ballot_sync(0xffffffffu, need);
        if (mneed) {
            unsigned long long b = 0;
            const int leader = __ffs(mneed) - 1;
            if (lane == leader) b = atomicAdd(q.take, (unsigned long long)__popc(mneed));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (need) {
                j = (int64_t)(b + __popc(mneed & lt));
                if (j >= n) {
                    exhausted = true;
                } else {
                    sim = q.i[4 * q.cap + j];
                    const SimDesc& S = kMulti ? sims[sim] : sS;
                    L.x[0] = q.f[0 * q.cap + j]; L.x[1] = q.f[1 * q.cap + j]; L.x[2] = q.f[2 * q.cap + j];
                    L.u[0] = q.f[3 * q.cap + j]; L.u[1] = q.f[4 * q.cap + j]; L.u[2] = q.f[5 * q.cap + j];
                    L.E = q.f[6 * q.cap + j];
                    L.t = q.t[j];
                    L.tf = 0.0f;
                    L.panel = q.i[0 * q.cap + j];
                    parn = q.i[1 * q.cap + j];
                    eid = q.i[2 * q.cap + j];
                    scat = q.i[3 * q.cap + j];
                    Pn = kMulti ? S.panels + L.panel * kPanelStride : sP + L.panel * kPanelStride;
                    pann = (int32_t)Pn[30];
                    if (entries) {
                        er.panel = L.panel;
                        er.y = L.x[1]; er.z = L.x[2];
                        er.ux = L.u[0]; er.uy = L.u[1]; er.uz = L.u[2];
                        er.E = L.E;
                    }
                    st_seed(rst, S.key0, S.key1, kTagDet + (uint32_t)(parn & 1), (uint32_t)eid, 0u);
                    nev = 0; nh = 0; step = 0; nsteps = 0;
                    overflow = false;
                    active = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, !active && exhausted)) break;
        // one Woodcock step in the panel (photonde, gPET_kernals.cu:1013-1193)
        bool done = false;
        unsigned capped = 0;
        if (active) {
            const SimDesc& S = kMulti ? sims[sim] : sS;
            nsteps++;
            do {   // a single pass: `break` ends the step
                float lammin = wck_at(S.wck_det, S.wck_e0, S.wck_ide, L.E);
                float s = -lammin * dm_logf(unif());
                L.x[0] = dm_fma(s, L.u[0], L.x[0]);
                L.x[1] = dm_fma(s, L.u[1], L.x[1]);
                L.x[2] = dm_fma(s, L.u[2], L.x[2]);
                L.tf = dm_fma(s, DM_INV_SPEED, L.tf);
                if (fabsf(L.x[1]) > Pn[1] * 0.5f || fabsf(L.x[2]) > Pn[2] * 0.5f || L.x[0] * Pn[18] < 0.0f ||
                    L.x[0] * Pn[18] > Pn[0]) {
                    done = true;
                    break;
                }
                int m_id = -1, M_id = -1, L_id = -1;
                crystal_search(S, Pn, L.x, m_id, M_id, L_id);
                float den = S.det_den[m_id];
                int mat = S.det_mat[m_id];
                float lamden = lammin * den;
                float4 xs = xs_at(S, mat, L.E);
                float prob = dm_fma(-lamden, xs.x, 1.0f);
                if (prob < 0.0f) prob = 0.0f;
                float rn = unif();
                if (rn < prob) break;   // virtual
                prob = dm_fma(lamden, xs.y, prob);
                int type = 0;
                float dep = 0.0f;
                if (rn < prob) {
                    float efrac, cost;
                    kn_sample_u(L.E, unif, efrac, cost);
                    float de = L.E * (1.0f - efrac);
                    float phi = unif();
                    if (m_id != 1) {   // a crystal (not the gap)
                        PEvent e;
                        e.modn = M_id; e.cryn = L_id;
                        e.E = de; e.t = L.t + (double)L.tf; e.x = L.x[0]; e.y = L.x[1]; e.z = L.x[2];
                        if (rec_hits) put_hit(M_id, L_id, 1, de, e.t);
                        if (!adder(ev, nev, e)) overflow = true;
                    }
                    L.E -= de;
                    if (L.E < S.eabsph) {
                        type = 2; dep = L.E;
                    } else {
                        rotate(L.u[0], L.u[1], L.u[2], cost, phi);
                        break;
                    }
                } else {
                    prob = dm_fma(lamden, xs.z, prob);
                    if (rn < prob) {
                        float cost = rayleigh_surface_u(S, L.E, mat, unif);
                        float phi = unif();
                        rotate(L.u[0], L.u[1], L.u[2], cost, phi);
                        break;
                    }
                    type = 4; dep = L.E;
                }
                if (m_id != 1) {   // a crystal (not the gap)
                    PEvent e;
                    e.modn = M_id; e.cryn = L_id;
                    e.E = dep; e.t = L.t + (double)L.tf; e.x = L.x[0]; e.y = L.x[1]; e.z = L.x[2];
                    if (rec_hits) put_hit(M_id, L_id, type, dep, e.t);
                    if (!adder(ev, nev, e)) overflow = true;
                }
                done = true;
            } while (false);
            step++;
            if (!done && step >= kMaxSteps) {
                done = true;
                capped = 1;
            }
            if (done) {
                if (nev) nev = readout(S, ev, nev);
                if (entries) {
                    er.crystal = nev ? ev[0].cryn : -1;
                    er.depth = nev ? ev[0].x * Pn[18] : 0.0f;
                    er.Edep = nev ? ev[0].E : 0.0f;
                    entries[j] = er;
                }
                t_steps.add(cnt, CF(det_steps), sim, nsteps);
                t_cap.add(cnt, CF(stepcap), sim, capped);
                t_over.add(cnt, CF(overflow), sim, overflow ? 1u : 0u);
                t_pulse.add(cnt, CF(n_pulse), sim, (unsigned)nev);
                t_hit.add(cnt, CF(n_hit), sim, rec_hits ? (unsigned)nh : 0u);
            }
        }
        // append the pulses and hits of the photons that finished, one atomic per warp
        if (!__any_sync(0xffffffffu, done)) continue;
        const int my_ev = done ? nev : 0;
        int inc = my_ev;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        int tot = __shfl_sync(0xffffffffu, inc, 31);
        if (tot) {
            unsigned long long b = 0;
            if (lane == 31) b = atomicAdd(P.count, (unsigned long long)tot);
            b = __shfl_sync(0xffffffffu, b, 31);
            unsigned long long o = b + (unsigned long long)(inc - my_ev);
            for (int i = 0; i < my_ev; ++i, ++o) {
                if (o >= (unsigned long long)P.cap) { n_pdrop++; continue; }
                P.parn[o] = parn; P.pann[o] = pann; P.modn[o] = ev[i].modn; P.cryn[o] = ev[i].cryn;
                P.siten[o] = site_of(kMulti ? sims[sim] : sS, pann, ev[i].modn, ev[i].cryn);
                P.eventid[o] = eid; P.t[o] = ev[i].t;
                P.E[o] = ev[i].E; P.x[o] = ev[i].x; P.y[o] = ev[i].y; P.z[o] = ev[i].z;
                P.meta[o] = (uint8_t)(i | (scat ? 0x80 : 0));
                if (P.sim) P.sim[o] = sim;
            }
        }
        if (done) active = false;
    }
    t_steps.flush(cnt, CF(det_steps));
    t_cap.flush(cnt, CF(stepcap));
    t_over.flush(cnt, CF(overflow));
    t_pulse.flush(cnt, CF(n_pulse));
    t_hit.flush(cnt, CF(n_hit));
    n_pdrop = warp_sum(n_pdrop); n_hdrop = warp_sum(n_hdrop);
    if (lane == 0) {
        if (n_pdrop) atomicAdd(&cnt->pulse_drop, n_pdrop);
        if (n_hdrop) atomicAdd(&cnt->hit_drop, n_hdrop);
    }
}

static bool valid_threads(unsigned t) { return t >= 32 && t <= 256 && t % 32 == 0; }

cudaError_t launch_source(bool multi, unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                          const Wave* waves, int wi, const PairBuf& pb, Counters* cnt)
{
    if (!valid_threads(threads)) return cudaErrorInvalidValue;
    if (multi) k_source<true><<<blocks, threads, smem, s>>>(waves, wi, pb, cnt);
    else k_source<false><<<blocks, threads, smem, s>>>(waves, wi, pb, cnt);
    return cudaGetLastError();
}

cudaError_t launch_walk(bool multi, unsigned blocks, cudaStream_t s, const Wave* waves, int wi, const PairBuf& pb)
{
    if (multi) k_walk<true><<<blocks, 256, 0, s>>>(waves, wi, pb);
    else k_walk<false><<<blocks, 256, 0, s>>>(waves, wi, pb);
    return cudaGetLastError();
}

cudaError_t walk_blocks_per_sm(bool multi, int* blocks)
{
    return multi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_walk<true>, 256, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_walk<false>, 256, 0);
}

cudaError_t launch_phantom(bool multi, unsigned blocks, size_t smem, cudaStream_t s, const Wave* waves, int wi,
                           const PairBuf& pb, const QueueDev& q, Counters* cnt, int period)
{
    if (period < 1 || period > 32) return cudaErrorInvalidValue;
    if (multi) k_phantom<true><<<blocks, 256, smem, s>>>(waves, wi, pb, q, cnt, period);
    else k_phantom<false><<<blocks, 256, smem, s>>>(waves, wi, pb, q, cnt, period);
    return cudaGetLastError();
}

cudaError_t launch_detector(bool multi, unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                            const SimDesc* sims, const QueueDev& q, const PulseDev& P, const HitDev& H, int rec_hits,
                            Counters* cnt, EntryRec* entries)
{
    if (!valid_threads(threads)) return cudaErrorInvalidValue;
    if (multi) k_detector<true><<<blocks, threads, smem, s>>>(sims, q, P, H, rec_hits, cnt, entries);
    else k_detector<false><<<blocks, threads, smem, s>>>(sims, q, P, H, rec_hits, cnt, entries);
    return cudaGetLastError();
}

cudaError_t phantom_blocks_per_sm(bool multi, size_t smem, int* blocks)
{
    return multi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_phantom<true>, 256, smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_phantom<false>, 256, smem);
}

cudaError_t detector_blocks_per_sm(bool multi, unsigned threads, size_t smem, int* blocks)
{
    if (!valid_threads(threads)) return cudaErrorInvalidValue;
    return multi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_detector<true>, (int)threads, smem)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_detector<false>, (int)threads, smem);
}

// shared-memory carveout of `f` just large enough for `blocks` resident
// blocks with `smem` dynamic bytes each, so that the rest of the SM's unified
// L1 / shared memory serves as L1 (k_phantom's spill reloads and table
// gathers); a hint the CUDA driver may round up
template <class F>
static cudaError_t set_carveout(F* f, int blocks, size_t smem)
{
    int dev = 0, per_sm = 0, reserved = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, f)) != cudaSuccess) return e;
    const size_t need = (size_t)blocks * (fa.sharedSizeBytes + smem + (size_t)reserved);
    int pct = per_sm > 0 ? (int)((100 * need + per_sm - 1) / (size_t)per_sm) : 100;
    pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
    return cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

// the panels staged in shared memory (single-simulation launches) can take
// the source, phantom and detector kernels above the 48 KB that need no opt-in
cudaError_t transport_set_smem(size_t smem)
{
    const int v = (int)smem;
    cudaError_t e;
    if ((e = set_carveout(k_phantom<false>, 5, smem)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_source<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(k_phantom<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v)) != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_detector<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}

cudaError_t transport_kernels_loadable()
{
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, k_phantom<false>);
}

template __global__ void k_source<false>(const Wave*, int, PairBuf, Counters*);
template __global__ void k_source<true>(const Wave*, int, PairBuf, Counters*);
template __global__ void k_walk<false>(const Wave*, int, PairBuf);
template __global__ void k_walk<true>(const Wave*, int, PairBuf);
template __global__ void k_phantom<false>(const Wave*, int, PairBuf, QueueDev, Counters*, int);
template __global__ void k_phantom<true>(const Wave*, int, PairBuf, QueueDev, Counters*, int);
template __global__ void k_detector<false>(const SimDesc*, QueueDev, PulseDev, HitDev, int, Counters*, EntryRec*);
template __global__ void k_detector<true>(const SimDesc*, QueueDev, PulseDev, HitDev, int, Counters*, EntryRec*);

}  // namespace gpet
