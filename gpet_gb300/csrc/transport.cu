// transport.cu - source, positron range, annihilation, phantom and detector
// transport kernels (the work of setPosition/setPositionForPhoton, photon and
// photonde in gPET_kernals.cu:256-1233), for sm_103a.
//
// Layout: one thread per decay runs the source stage and both photons through
// the phantom; photons that reach a panel are compacted (warp ballot, one
// atomic per warp) into a structure-of-arrays detector queue. A second kernel
// runs one thread per queued photon through the panel, applies the per-photon
// adder and readout, and appends pulses and hits (one atomic per warp).
#include "kernels.h"

namespace gpet {

__device__ __forceinline__ void load_sim(const SimDesc* __restrict__ g, SimDesc& s, float* sP)
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(g);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&s);
    for (int i = threadIdx.x; i < (int)(sizeof(SimDesc) / 4); i += blockDim.x) dst[i] = src[i];
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

// source stage of one decay (setPosition gPET_kernals.cu:483-561 for a source
// in the H3 form: the decay's source is fixed by its index, its time is a
// truncated exponential on [0, dt)); PSF records (setPositionForPhoton
// :563-604, with the second photon's time set) when npsf > 0.
// Returns how many photons of the pair exist (0, 1 or 2).
__device__ int sample_decay(const SimDesc& S, int64_t d, Photon ph[2])
{
    Stream st;
    st_init(st, S.key0, S.key1, kTagDecay, (uint64_t)d);
    if (S.npsf > 0) {
        const double* r = S.psf + 8 * d;
        if (S.psf_ptype == 1) {
            ph[0].x[0] = (float)r[0]; ph[0].x[1] = (float)r[1]; ph[0].x[2] = (float)r[2];
            ph[0].u[0] = (float)r[4]; ph[0].u[1] = (float)r[5]; ph[0].u[2] = (float)r[6];
            ph[0].E = (float)r[7]; ph[0].t = r[3]; ph[0].nscat = 0;
            return (r[3] > 0.0 && ph[0].E >= 0.0f) ? 1 : 0;
        }
        float pos[3] = {(float)r[0], (float)r[1], (float)r[2]};
        float dir[3] = {(float)r[4], (float)r[5], (float)r[6]};
        if (S.useprange) positron_range(S, pos, (float)r[7], dir, st);
        make_pair(S, st, pos, r[3], ph);
        return 2;
    }
    int si = 0;
    while (si < S.nsrc - 1 && d >= S.src_end[si]) si++;
    double ud = st_ud(st);
    double tdec = -S.src_tau[si] * dm_log(1.0 - ud * S.src_cfac[si]);
    double t_us = (S.tstart_s + tdec) * 1e6;
    float br = st_u(st);
    if (!(br < S.iso_ratio[si])) return 0;
    float pos[3];
    shape_position(S, si, st, pos);
    if (S.useprange) {
        float ek = sample_ek(S.iso_coef[si], st);
        positron_range(S, pos, ek, nullptr, st);
    }
    make_pair(S, st, pos, t_us, ph);
    return 2;
}

__global__ void __launch_bounds__(256) k_source_phantom(const SimDesc* __restrict__ gS, int64_t d_begin,
                                                        int64_t d_end, QueueDev q, ExitRec* exits,
                                                        Counters* cnt)
{
    __shared__ SimDesc S;
    extern __shared__ float sP[];
    load_sim(gS, S, sP);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const unsigned lt = lanemask_lt();
    const int lane = threadIdx.x & 31;
    unsigned long long n_pairs = 0, n_entered = 0, n_steps = 0, n_cap = 0, n_drop = 0;
    for (int64_t base = d_begin + (int64_t)blockIdx.x * blockDim.x; base < d_end; base += stride) {
        const int64_t d = base + threadIdx.x;
        const bool valid = d < d_end;
        Photon ph[2];
        int nph = 0;
        if (valid) nph = sample_decay(S, d, ph);
        if (nph == 2) n_pairs++;
#pragma unroll 1
        for (int k = 0; k < 2; ++k) {
            Local L;
            bool entered = false;
            int status = 2;
            if (valid && k < nph) {
                Stream st;
                st_init(st, S.key0, S.key1, kTagPhantom + k, (uint64_t)d);
                int steps = 0;
                status = phantom_transport(S, ph[k], st, steps);
                n_steps += steps;
                if (status == 3) n_cap++;
                if (status == 1) entered = enter_panel(sP, S.npanels, ph[k], L);
            }
            const unsigned m = __ballot_sync(0xffffffffu, entered);
            if (m) {
                unsigned long long b = 0;
                const int leader = __ffs(m) - 1;
                if (lane == leader) b = atomicAdd(q.count, (unsigned long long)__popc(m));
                b = __shfl_sync(0xffffffffu, b, leader);
                if (entered) {
                    const unsigned long long j = b + __popc(m & lt);
                    if (j < (unsigned long long)q.cap) {
                        q.f[0 * q.cap + j] = L.x[0];
                        q.f[1 * q.cap + j] = L.x[1];
                        q.f[2 * q.cap + j] = L.x[2];
                        q.f[3 * q.cap + j] = L.u[0];
                        q.f[4 * q.cap + j] = L.u[1];
                        q.f[5 * q.cap + j] = L.u[2];
                        q.f[6 * q.cap + j] = L.E;
                        q.t[j] = L.t;
                        q.i[0 * q.cap + j] = L.panel;
                        q.i[1 * q.cap + j] = (int32_t)(2 * d + k);
                        q.i[2 * q.cap + j] = (int32_t)d;
                        q.i[3 * q.cap + j] = ph[k].nscat;
                        n_entered++;
                    } else {
                        n_drop++;
                    }
                }
            }
            if (exits && valid) {
                ExitRec e;
                if (k < nph) {
                    e.x = ph[k].x[0]; e.y = ph[k].x[1]; e.z = ph[k].x[2];
                    e.ux = ph[k].u[0]; e.uy = ph[k].u[1]; e.uz = ph[k].u[2];
                    e.E = ph[k].E; e.nscat = ph[k].nscat; e.t = ph[k].t;
                } else {
                    e.x = e.y = e.z = e.ux = e.uy = e.uz = e.E = 0.0f; e.nscat = 0; e.t = 0.0;
                }
                e.status = status;
                e.panel = entered ? L.panel : -1;
                exits[2 * (d - d_begin) + k] = e;
            }
        }
    }
    n_pairs = warp_sum(n_pairs); n_entered = warp_sum(n_entered); n_steps = warp_sum(n_steps);
    n_cap = warp_sum(n_cap); n_drop = warp_sum(n_drop);
    if (lane == 0) {
        if (n_pairs) atomicAdd(&cnt->pairs, n_pairs);
        if (n_entered) atomicAdd(&cnt->entered, n_entered);
        if (n_steps) atomicAdd(&cnt->ph_steps, n_steps);
        if (n_cap) atomicAdd(&cnt->stepcap, n_cap);
        if (n_drop) atomicAdd(&cnt->queue_drop, n_drop);
    }
}

// ------------------------------------------------------------- detector
struct PEvent {
    int32_t pann, modn, cryn, siten;
    double t;
    float E, x, y, z;
};

// adder, gPET_kernals.cu:737-755
__device__ __forceinline__ bool adder(PEvent* ev, int& n, const PEvent& e)
{
    for (int i = 0; i < n; ++i) {
        if (e.siten == ev[i].siten) {
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
    for (int i = 0; i < n; ++i) {
        if (depth == 0) ev[i].siten = 0;
        else if (depth == 1) ev[i].siten = ev[i].pann;
        else if (depth == 2) ev[i].siten = ev[i].pann * S.moduleN + ev[i].modn;
    }
    unsigned dead = 0;
    int k = 0;
    for (int i = 0; i < n; ++i) {
        if (dead & (1u << i)) continue;
        PEvent e0 = ev[i];
        for (int j = i + 1; j < n; ++j) {
            const PEvent e = ev[j];
            if (e.siten == e0.siten) {   // one photon: parn always equal
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

__global__ void __launch_bounds__(256) k_detector(const SimDesc* __restrict__ gS, QueueDev q, PulseDev P,
                                                  HitDev H, int rec_hits, Counters* cnt)
{
    __shared__ SimDesc S;
    extern __shared__ float sP[];
    load_sim(gS, S, sP);
    unsigned long long nq = *q.count;
    if (nq > (unsigned long long)q.cap) nq = (unsigned long long)q.cap;
    const int64_t n = (int64_t)nq;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    unsigned long long n_steps = 0, n_over = 0, n_cap = 0, n_pdrop = 0, n_hdrop = 0;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t j = base + threadIdx.x;
        const bool valid = j < n;
        PEvent ev[kMaxPulse];
        int nev = 0;
        int nh = 0;
        int32_t hid[kMaxHits][4];
        float hf[kMaxHits][5];
        int32_t parn = 0, eid = 0, scat = 0;
        bool overflow = false;
        if (valid) {
            Local L;
            L.x[0] = q.f[0 * q.cap + j]; L.x[1] = q.f[1 * q.cap + j]; L.x[2] = q.f[2 * q.cap + j];
            L.u[0] = q.f[3 * q.cap + j]; L.u[1] = q.f[4 * q.cap + j]; L.u[2] = q.f[5 * q.cap + j];
            L.E = q.f[6 * q.cap + j];
            L.t = q.t[j];
            L.panel = q.i[0 * q.cap + j];
            parn = q.i[1 * q.cap + j];
            eid = q.i[2 * q.cap + j];
            scat = q.i[3 * q.cap + j];
            const float* Pn = sP + L.panel * kPanelStride;
            const int32_t pann = (int32_t)Pn[30];
            Stream st;
            st_init(st, S.key0, S.key1, kTagDet + (parn & 1), (uint64_t)(uint32_t)eid);
            // photonde transport loop, gPET_kernals.cu:1013-1193
            int step;
            for (step = 0; step < kMaxSteps; ++step) {
                n_steps++;
                float lammin = wck_at(S.wck_det, S.wck_e0, S.wck_ide, L.E);
                float s = -lammin * dm_logf(st_u(st));
                L.x[0] += s * L.u[0];
                L.x[1] += s * L.u[1];
                L.x[2] += s * L.u[2];
                L.t += (double)s / kSpe;
                if (fabsf(L.x[1]) > Pn[1] * 0.5f || fabsf(L.x[2]) > Pn[2] * 0.5f || L.x[0] * Pn[18] < 0.0f ||
                    L.x[0] * Pn[18] > Pn[0])
                    break;
                int m_id = -1, M_id = -1, L_id = -1;
                crystal_search(S, Pn, L.x, m_id, M_id, L_id);
                float den = S.det_den[m_id];
                int mat = S.det_mat[m_id];
                float lamden = lammin * den;
                float4 xs = xs_at(S, mat, L.E);
                float prob = 1.0f - lamden * xs.x;
                if (prob < 0.0f) prob = 0.0f;
                float rn = st_u(st);
                if (rn < prob) continue;
                prob += lamden * xs.y;
                int type = 0;
                float dep = 0.0f;
                if (rn < prob) {
                    float efrac, cost;
                    kn_sample(L.E, st, efrac, cost);
                    float de = L.E * (1.0f - efrac);
                    float phi = st_u(st);
                    if (m_id == 0) {
                        PEvent e;
                        e.pann = pann; e.modn = M_id; e.cryn = L_id;
                        e.siten = pann * S.moduleN * S.crystalN + M_id * S.crystalN + L_id;
                        e.E = de; e.t = L.t; e.x = L.x[0]; e.y = L.x[1]; e.z = L.x[2];
                        if (rec_hits) {
                            if (nh < kMaxHits) {
                                hid[nh][0] = pann; hid[nh][1] = M_id; hid[nh][2] = L_id; hid[nh][3] = 1;
                                hf[nh][0] = de; hf[nh][1] = (float)L.t; hf[nh][2] = L.x[0]; hf[nh][3] = L.x[1];
                                hf[nh][4] = L.x[2];
                                nh++;
                            } else {
                                overflow = true;
                            }
                        }
                        if (!adder(ev, nev, e)) overflow = true;
                    }
                    L.E -= de;
                    if (L.E < S.eabsph) {
                        type = 2; dep = L.E;
                    } else {
                        rotate(L.u[0], L.u[1], L.u[2], cost, phi);
                        continue;
                    }
                } else {
                    prob += lamden * xs.z;
                    if (rn < prob) {
                        float cost = rayleigh_surface(S, L.E, mat, st);
                        float phi = st_u(st);
                        rotate(L.u[0], L.u[1], L.u[2], cost, phi);
                        continue;
                    }
                    type = 4; dep = L.E;
                }
                if (m_id == 0) {
                    PEvent e;
                    e.pann = pann; e.modn = M_id; e.cryn = L_id;
                    e.siten = pann * S.moduleN * S.crystalN + M_id * S.crystalN + L_id;
                    e.E = dep; e.t = L.t; e.x = L.x[0]; e.y = L.x[1]; e.z = L.x[2];
                    if (rec_hits) {
                        if (nh < kMaxHits) {
                            hid[nh][0] = pann; hid[nh][1] = M_id; hid[nh][2] = L_id; hid[nh][3] = type;
                            hf[nh][0] = dep; hf[nh][1] = (float)L.t; hf[nh][2] = L.x[0]; hf[nh][3] = L.x[1];
                            hf[nh][4] = L.x[2];
                            nh++;
                        } else {
                            overflow = true;
                        }
                    }
                    if (!adder(ev, nev, e)) overflow = true;
                }
                break;
            }
            if (step == kMaxSteps) n_cap++;
            if (nev) nev = readout(S, ev, nev);
            if (overflow) n_over++;
        }
        // append pulses and hits, one atomic per warp
        int inc = nev;
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
            unsigned long long o = b + (unsigned long long)(inc - nev);
            for (int i = 0; i < nev; ++i, ++o) {
                if (o >= (unsigned long long)P.cap) { n_pdrop++; continue; }
                P.parn[o] = parn; P.pann[o] = ev[i].pann; P.modn[o] = ev[i].modn; P.cryn[o] = ev[i].cryn;
                P.siten[o] = ev[i].siten; P.eventid[o] = eid; P.t[o] = ev[i].t;
                P.E[o] = ev[i].E; P.x[o] = ev[i].x; P.y[o] = ev[i].y; P.z[o] = ev[i].z;
                P.meta[o] = (uint8_t)(i | (scat ? 0x80 : 0));
            }
        }
        if (rec_hits) {
            int hinc = nh;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, hinc, o);
                if (lane >= o) hinc += v;
            }
            int htot = __shfl_sync(0xffffffffu, hinc, 31);
            if (htot) {
                unsigned long long b = 0;
                if (lane == 31) b = atomicAdd(H.count, (unsigned long long)htot);
                b = __shfl_sync(0xffffffffu, b, 31);
                unsigned long long o = b + (unsigned long long)(hinc - nh);
                for (int i = 0; i < nh; ++i, ++o) {
                    if (o >= (unsigned long long)H.cap) { n_hdrop++; continue; }
                    H.id[5 * o + 0] = parn;
                    H.id[5 * o + 1] = hid[i][0]; H.id[5 * o + 2] = hid[i][1]; H.id[5 * o + 3] = hid[i][2];
                    H.id[5 * o + 4] = hid[i][3];
                    for (int c = 0; c < 5; ++c) H.f[5 * o + c] = hf[i][c];
                }
            }
        }
    }
    n_steps = warp_sum(n_steps); n_over = warp_sum(n_over); n_cap = warp_sum(n_cap);
    n_pdrop = warp_sum(n_pdrop); n_hdrop = warp_sum(n_hdrop);
    if (lane == 0) {
        if (n_steps) atomicAdd(&cnt->det_steps, n_steps);
        if (n_over) atomicAdd(&cnt->overflow, n_over);
        if (n_cap) atomicAdd(&cnt->stepcap, n_cap);
        if (n_pdrop) atomicAdd(&cnt->pulse_drop, n_pdrop);
        if (n_hdrop) atomicAdd(&cnt->hit_drop, n_hdrop);
    }
}

}  // namespace gpet
