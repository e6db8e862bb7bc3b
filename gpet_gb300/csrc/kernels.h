// kernels.h - device buffers and kernel entry points shared by the host
// runtime (gpet_api.cpp) and the kernel translation units.
#pragma once
#include <cstddef>

#include "device.cuh"

namespace gpet {

// phantom exit record (48 bytes), one per photon slot
struct ExitRec {
    float x, y, z, ux, uy, uz, E;
    int32_t nscat;
    double t;
    int32_t status, panel;
};

// an emitted photon (source phase space, gPET.cu:63-87), 40 bytes; t = 0
// when the photon slot carries nothing
struct SrcRec {
    float x, y, z, ux, uy, uz, E;
    int32_t eventid;
    double t;
};
static_assert(sizeof(SrcRec) == 40, "source record is 40 bytes");

// A wave of decays: global indices [g0[i], g0[i+1]) are decays d0[i] ..
// of simulation sim[i] (sims[] in device memory). Waves live in a device
// table that the kernels index, so that the launches of a chunk of waves do
// not change from chunk to chunk (one CUDA graph serves them all).
constexpr int kMaxSeg = 128;
struct Wave {
    const SimDesc* sims;
    const int64_t* g0;            // [nseg + 1]
    const int64_t* d0;            // [nseg]
    const int32_t* sim;           // [nseg]
    int32_t nseg;
    int64_t n;                    // decays in the wave
    unsigned long long* work;     // photon counter of k_phantom, zero at launch
    unsigned long long* walkn;    // [kWalkLists] entries of the positron walk lists, zero at launch
    ExitRec* exits;               // per photon of the wave, or NULL
    SrcRec* source;               // per photon of the wave, or NULL
};

// detector queue, structure of arrays (cap entries each)
struct QueueDev {
    float* f;                     // [7][cap]: local x, y, z, ux, uy, uz, E
    double* t;                    // [cap]
    int32_t* i;                   // [5][cap]: panel index, parn, event id, phantom scatters, simulation
    unsigned long long* count;
    int64_t cap;
    unsigned long long* take = nullptr;   // next entry for the detector stage's lanes (zero before it)
};

// pulses after adder + readout, structure of arrays
struct PulseDev {
    int32_t *parn, *pann, *modn, *cryn, *siten, *eventid;
    double* t;
    float *E, *x, *y, *z;
    uint8_t* meta;                // slot | 0x80 if the photon scattered in the phantom
    int32_t* sim;                 // simulation of each pulse (NULL: all simulation 0)
    unsigned long long* count;
    int64_t cap;
};

struct HitDev {
    int32_t* id;                  // [cap][5]
    float* f;                     // [cap][5]
    int32_t* sim;                 // [cap] (may be NULL)
    unsigned long long* count;
    int64_t cap;
};

struct Counters {
    unsigned long long pairs, entered, stepcap, ph_steps, det_steps, overflow, pulse_drop, hit_drop, queue_drop;
    unsigned long long n_thr, n_dead, n_single, n_coinc, n_true, n_scat, n_rand, n_mult;
    unsigned long long n_pulse, n_hit;
    unsigned long long n_surrogate;   // photons whose response came from the surrogate
    unsigned long long n_noise;       // background singles added before the digitizer
};

// a photon entering a panel and its detector response after adder and
// readout (training data of the surrogate), 40 bytes
struct EntryRec {
    int32_t panel;
    float y, z, ux, uy, uz, E;    // entry point and direction (panel-local), energy (eV)
    int32_t crystal;              // crystal of its first pulse, -1: no pulse
    float depth;                  // depth of that pulse below the entry face (cm)
    float Edep;                   // its energy (eV)
};
static_assert(sizeof(EntryRec) == 40, "entry record is 40 bytes");

// cnt[sim].field += v, lanes of a warp grouped by simulation (all lanes of the
// warp must call it together)
__device__ __forceinline__ void add_by_sim(Counters* cnt, int sim, int field, unsigned v)
{
    const unsigned peers = __match_any_sync(0xffffffffu, sim);
    const unsigned tot = __reduce_add_sync(peers, v);
    if (tot && (threadIdx.x & 31) == __ffs(peers) - 1)
        atomicAdd(reinterpret_cast<unsigned long long*>(cnt + sim) + field, (unsigned long long)tot);
}

#define CF(name) ((int)(offsetof(Counters, name) / sizeof(unsigned long long)))

// per-thread counter for the simulation the thread is working on; flushed
// when the simulation changes (rare: waves are contiguous per simulation) and
// once per warp at the end
struct SimTally {
    int sim = -1;
    unsigned v = 0;
    __device__ __forceinline__ void add(Counters* cnt, int field, int s, unsigned x)
    {
        if (s != sim) {
            if (v) atomicAdd(reinterpret_cast<unsigned long long*>(cnt + sim) + field, (unsigned long long)v);
            sim = s;
            v = 0;
        }
        v += x;
    }
    __device__ __forceinline__ void flush(Counters* cnt, int field)
    {
        add_by_sim(cnt, sim < 0 ? 0 : sim, field, v);
        v = 0;
    }
};

// digitizer parameters (main.cu:158-182 plus the coincidence sorter)
struct DigiParams {
    uint32_t key0, key1;
    int32_t blurpolicy;
    float Eref, Rref, Eslope, Sblur, Eth;
    int32_t dlevel, dtype;
    double tau;                   // dead time, us
    float ewin_lo, ewin_hi;
    double window;                // coincidence window, us
    int32_t coinc_policy;
    int32_t moduleN, crystalN;
};

// emitted pairs of a sub-chunk of decays, structure of arrays
constexpr int kWalkLists = 4;    // positron walk lists by estimated length
constexpr int kWalkFields = 8;   // floats per walk: start (3), displacement (3), its length, length covered

struct PairBuf {
    float* f;                     // [11][cap]: x, y, z, u0 (3), u1 (3), E0, E1
    double* t;                    // [cap]
    uint8_t* nph;                 // [cap]: photons emitted (0, 1 or 2)
    float* wf;                    // walk lists [kWalkLists][kWalkFields][cap]
    int32_t* wj;                  // walk lists [kWalkLists][cap]: the decay's index within the wave
    int64_t cap;
};

// Counters is an array indexed by simulation; kMulti selects per-thread
// simulation descriptors (several simulations in one wave)
// waves[wi] is the wave to process. period: k_phantom takes its staged
// finished photons through the panel search once at least `period` (1..32)
// are waiting
template <bool kMulti> __global__ void k_source(const Wave* waves, int wi, PairBuf pb, Counters* cnt);
template <bool kMulti>
__global__ void k_phantom(const Wave* waves, int wi, PairBuf pb, QueueDev q, Counters* cnt, int period);
template <bool kMulti>
__global__ void k_detector(const SimDesc* sims, QueueDev q, PulseDev P, HitDev H, int rec_hits, Counters* cnt,
                           EntryRec* entries);

// host-side launchers (transport.cu): `multi` picks the kMulti instance,
// smem is the dynamic shared memory (panels of the one simulation, or 0);
// threads per block: a multiple of 32 up to 256 (k_phantom: 256)
cudaError_t launch_source(bool multi, unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                          const Wave* waves, int wi, const PairBuf& pb, Counters* cnt);
// the wave's deferred positron-range walks (after k_source, before k_phantom)
cudaError_t launch_walk(bool multi, unsigned blocks, cudaStream_t s, const Wave* waves, int wi, const PairBuf& pb);
cudaError_t walk_blocks_per_sm(bool multi, int* blocks);
cudaError_t launch_phantom(bool multi, unsigned blocks, size_t smem, cudaStream_t s, const Wave* waves, int wi,
                           const PairBuf& pb, const QueueDev& q, Counters* cnt, int period);
// entries: one record per queue entry (or NULL)
cudaError_t launch_detector(bool multi, unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                            const SimDesc* sims, const QueueDev& q, const PulseDev& P, const HitDev& H, int rec_hits,
                            Counters* cnt, EntryRec* entries);
// resident k_phantom blocks per SM at 256 threads and `smem` bytes
cudaError_t phantom_blocks_per_sm(bool multi, size_t smem, int* blocks);
cudaError_t transport_set_smem(size_t smem);
cudaError_t detector_blocks_per_sm(bool multi, unsigned threads, size_t smem, int* blocks);
// cudaSuccess when the transport kernels have an image for the current device
cudaError_t transport_kernels_loadable();

// ---- digitizer building blocks (digitizer.cu), all stream-ordered
struct DigiScratch {
    // per-pulse working arrays (capacity cap)
    uint32_t *idx_a, *idx_b;      // index permutations
    uint64_t *key_a, *key_b;      // sort keys
    uint32_t* torder;             // pulse index in time order
    uint32_t* flags;              // per pulse: bit0 alive after dead time
    int32_t* site;                // dead-time site per pulse
    uint32_t* hist;               // radix histograms / scan scratch
    uint32_t* scan_aux;
    uint32_t* sel;                // compaction output
    float *Eb, *xb, *yb, *zb;     // blurred energy and position per pulse
    int64_t cap, hist_cap;
    // outputs
    uint32_t* single_idx;         // pulse index of each single, time order
    int64_t* coinc_pairs;         // [coinc_cap][2] single indices
    uint8_t* coinc_class;
    uint32_t* wcount;             // per-single pair count / offsets
    uint32_t* wend;               // per window start: one past its last single
    int64_t coinc_cap;
    unsigned long long* dcount;   // device counters: [0] selected, [1] singles, [2] coinc
};

// the reference's Event record, 48 bytes (gPET.h:87-92)
struct EventRec {
    int32_t parn, pann, modn, cryn, siten, eventid;
    double t;
    float E, x, y, z;
};
static_assert(sizeof(EventRec) == 48, "Event record is 48 bytes");

int gather_events(const PulseDev& P, const uint32_t* idx, int64_t n, bool blurred, const DigiScratch& D,
                  EventRec* out, uint8_t* meta, cudaStream_t s);
// the blurred records written straight into mapped (pinned) host memory seen
// through its device address (16-byte aligned), flags[j] = scattered in the
// phantom (may be null)
// max_blocks > 0 caps the grid (a gather that runs beside other kernels)
int gather_events_mapped(const PulseDev& P, const uint32_t* idx, int64_t n, const DigiScratch& D, EventRec* out,
                         uint8_t* flags, cudaStream_t s, unsigned max_blocks = 0);

// digitizer kernels (digitizer.cu), for callers that orchestrate them with
// their own working memory
constexpr int kDigiTile = 4096;   // items per block of the radix and scan kernels
__global__ void k_scan_reduce(const uint32_t* in, int64_t n, uint32_t* aux);
__global__ void k_scan_aux(uint32_t* aux, int64_t nb, uint32_t* total);
__global__ void k_scan_down(const uint32_t* in, int64_t n, const uint32_t* aux, uint32_t* out);
__global__ void k_radix_hist(const uint64_t* keys, int64_t n, int shift, uint32_t* hist, int64_t nblocks);
__global__ void k_radix_scatter(const uint64_t* kin, const uint32_t* vin, int64_t n, int shift, const uint32_t* off,
                                int64_t nblocks, uint64_t* kout, uint32_t* vout);
__global__ void k_blur_threshold(PulseDev P, int64_t n, const DigiParams* prms, float* Eb, float* xb, float* yb,
                                 float* zb, int32_t* site, uint32_t* sel, unsigned long long* nsel,
                                 unsigned long long* range);
__global__ void k_tie_fix(const uint64_t* key, uint32_t* idx, int64_t m, const double* t, const int32_t* parn,
                          const uint8_t* meta);
// host side of the sorts: stable LSD radix sort by bits [0, nbits) (8 per
// pass; result in ka, va), the time keys of the selected pulses (returns the
// key width), the site key width for sites up to smax
void radix_sort(uint64_t*& ka, uint32_t*& va, uint64_t*& kb, uint32_t*& vb, int64_t n, int nbits, uint32_t* hist,
                uint32_t* aux, uint32_t* total, cudaStream_t s, int64_t* launches);
int launch_time_keys(const uint32_t* sel, int64_t m, const double* t, const unsigned long long* range,
                     uint64_t* key, uint32_t* val, cudaStream_t s);
int site_key_bits(unsigned long long smax);
__global__ void k_site_keys(const uint32_t* torder, int64_t m, const int32_t* site, const int32_t* psim,
                            uint64_t* key, uint32_t* val);
__global__ void k_deadtime(const uint32_t* sorder, const uint64_t* skey, int64_t m, const double* t,
                           const DigiParams* prms, int multi, uint32_t* flags, Counters* cnt);
__global__ void k_window_pred(const uint32_t* torder, int64_t m, const uint32_t* flags, const float* Eb,
                              const int32_t* psim, const DigiParams* prms, uint32_t* pred, Counters* cnt);
__global__ void k_count_by_sim(const uint32_t* order, int64_t m, const int32_t* psim, Counters* cnt, int field);
__global__ void k_compact(const uint32_t* torder, const uint32_t* pred, const uint32_t* off, int64_t m,
                          uint32_t* out);
__global__ void k_coinc_count(const uint32_t* sidx, int64_t s, const double* t, const int32_t* pann,
                              const int32_t* psim, const DigiParams* prms, uint32_t* wcount, uint32_t* wend,
                              Counters* cnt);
__global__ void k_coinc_write(const uint32_t* sidx, int64_t s, const uint32_t* wend, const uint32_t* off,
                              const int32_t* pann, const int32_t* eid, const uint8_t* meta, const int32_t* psim,
                              const DigiParams* prms, int64_t* pairs, uint8_t* klass, int64_t cap, Counters* cnt);
__global__ void k_gather_events(PulseDev P, const uint32_t* idx, int64_t n, int blurred, const float* Eb,
                                const float* xb, const float* yb, const float* zb, const int32_t* site,
                                EventRec* out, uint8_t* meta);

// Background singles (addnoise, gPET_kernals.cu:699-735; never launched by
// the reference): a Poisson process over [t0, t1) us cut into intervals of
// interval_us, each drawn from its own stream (tag 9, id = interval):
// exponential gaps of mean lambda_us, energy N(emean, sigma), uniform panel,
// module and crystal, x/y/z uniform in (0, 1) as in the reference, parn and
// eventid -1. They skip the blur and are never "the same decay".
struct NoiseParams {
    uint32_t key0, key1;
    float lambda_us, emean, sigma;
    double t0_us, t1_us, interval_us;
    int64_t nint;
    int32_t npanels, moduleN, crystalN, sim;
};
constexpr int kMaxNoisePerInterval = 4096;
// events per interval into D.sel, their exclusive prefix into D.wcount, the
// total into *total_out (synchronises the stream); D.cap >= nint
int noise_count(const NoiseParams& np, DigiScratch& D, cudaStream_t s, int64_t* launches, int64_t* total_out);
// write them into P from index `base` on (after noise_count)
int noise_write(const NoiseParams& np, const DigiScratch& D, const PulseDev& P, int64_t base, Counters* cnt,
                cudaStream_t s, int64_t* launches);

// List-mode coincidences -> sinogram (single-slice rebinning): each pair's
// line between the two singles' global positions (blurred, panel-local ->
// global with the panel axes) gives angle phi in [0, pi), signed distance s
// from the axis and mean z; hist[(iz * n_phi + iphi) * n_s + is] counts the
// pairs whose class bit is set in class_mask (1 true, 2 scatter, 4 random).
struct SinoParams {
    int32_t n_s, n_phi, n_z;
    float s_max, z_max;
    int32_t class_mask;
};
int sinogram_device(const int64_t* pairs, const uint8_t* klass, int64_t c0, int64_t nc, const uint32_t* single_idx,
                    const DigiScratch& D, const int32_t* pann, const float* panels, const int32_t* id2panel,
                    int32_t nid, SinoParams sp, uint32_t* hist, cudaStream_t s);

// Runs blur .. coincidences on n pulses already in P (device), stream-ordered;
// returns 0 or a GPET_ERR code. Pulses of nsims simulations (P.sim) are
// digitized in one pass with parameters d_prms[sim] (device); singles come out
// in (simulation, t) order in D.single_idx, coincidences in D.coinc_*,
// per-simulation counts in d_cnt[sim]. `launches` accumulates kernel launches.
// D.dcount needs 16 entries.
int digitize_device(const PulseDev& P, int64_t n, const DigiParams* d_prms, int nsims, DigiScratch& D,
                    Counters* d_cnt, cudaStream_t s, int64_t* launches, int64_t* n_singles_out, int64_t* n_coinc_out);

}  // namespace gpet
