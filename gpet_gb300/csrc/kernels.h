// kernels.h - device buffers and kernel entry points shared by the host
// runtime (gpet_api.cpp) and the kernel translation units.
#pragma once
#include "device.cuh"

namespace gpet {

// detector queue, structure of arrays (cap entries each)
struct QueueDev {
    float* f;                     // [7][cap]: local x, y, z, ux, uy, uz, E
    double* t;                    // [cap]
    int32_t* i;                   // [4][cap]: panel index, parn, event id, phantom scatters
    unsigned long long* count;
    int64_t cap;
};

// pulses after adder + readout, structure of arrays
struct PulseDev {
    int32_t *parn, *pann, *modn, *cryn, *siten, *eventid;
    double* t;
    float *E, *x, *y, *z;
    uint8_t* meta;                // slot | 0x80 if the photon scattered in the phantom
    unsigned long long* count;
    int64_t cap;
};

struct HitDev {
    int32_t* id;                  // [cap][5]
    float* f;                     // [cap][5]
    unsigned long long* count;
    int64_t cap;
};

struct Counters {
    unsigned long long pairs, entered, stepcap, ph_steps, det_steps, overflow, pulse_drop, hit_drop, queue_drop;
    unsigned long long n_thr, n_dead, n_single, n_coinc, n_true, n_scat, n_rand, n_mult;
};

// phantom exit record (48 bytes), one per photon slot
struct ExitRec {
    float x, y, z, ux, uy, uz, E;
    int32_t nscat;
    double t;
    int32_t status, panel;
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
struct PairBuf {
    float* f;                     // [11][cap]: x, y, z, u0 (3), u1 (3), E0, E1
    double* t;                    // [cap]
    uint8_t* nph;                 // [cap]: photons emitted (0, 1 or 2)
    int64_t cap;
};

__global__ void k_source(const SimDesc* __restrict__ gS, int64_t d0, int64_t n, PairBuf pb, Counters* cnt);
__global__ void k_phantom(const SimDesc* __restrict__ gS, int64_t d0, int64_t nd, PairBuf pb,
                          unsigned long long* work, QueueDev q, ExitRec* exits, Counters* cnt);
__global__ void k_detector(const SimDesc* __restrict__ gS, QueueDev q, PulseDev P, HitDev H, int rec_hits,
                           Counters* cnt);

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
    int64_t* coinc_pairs;         // [2][coinc_cap] single indices
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

// digitizer kernels (digitizer.cu), for callers that orchestrate them with
// their own working memory
constexpr int kDigiTile = 4096;   // items per block of the radix and scan kernels
__global__ void k_scan_reduce(const uint32_t* in, int64_t n, uint32_t* aux);
__global__ void k_scan_aux(uint32_t* aux, int64_t nb, uint32_t* total);
__global__ void k_scan_down(const uint32_t* in, int64_t n, const uint32_t* aux, uint32_t* out);
__global__ void k_radix_hist(const uint64_t* keys, int64_t n, int shift, uint32_t* hist, int64_t nblocks);
__global__ void k_radix_scatter(const uint64_t* kin, const uint32_t* vin, int64_t n, int shift, const uint32_t* off,
                                int64_t nblocks, uint64_t* kout, uint32_t* vout);
__global__ void k_blur_threshold(PulseDev P, int64_t n, DigiParams prm, float* Eb, float* xb, float* yb, float* zb,
                                 int32_t* site, uint32_t* sel, unsigned long long* nsel);
__global__ void k_time_keys(const uint32_t* sel, int64_t m, const double* t, uint64_t* key, uint32_t* val);
__global__ void k_tie_fix(const uint64_t* key, uint32_t* idx, int64_t m, const int32_t* parn, const uint8_t* meta);
__global__ void k_site_keys(const uint32_t* torder, int64_t m, const int32_t* site, uint64_t* key, uint32_t* val);
__global__ void k_deadtime(const uint32_t* sorder, int64_t m, const int32_t* site, const double* t, double tau,
                           int dtype, uint32_t* flags, unsigned long long* nalive);
__global__ void k_window_pred(const uint32_t* torder, int64_t m, const uint32_t* flags, const float* Eb, float lo,
                              float hi, uint32_t* pred);
__global__ void k_compact(const uint32_t* torder, const uint32_t* pred, const uint32_t* off, int64_t m,
                          uint32_t* out);
__global__ void k_coinc_count(const uint32_t* sidx, int64_t s, const double* t, const int32_t* pann, double W,
                              int policy, uint32_t* wcount, uint32_t* wend, unsigned long long* nmult);
__global__ void k_coinc_write(const uint32_t* sidx, int64_t s, const uint32_t* wend, const uint32_t* off,
                              const int32_t* pann, const int32_t* eid, const uint8_t* meta, int policy,
                              int64_t* pairs, uint8_t* klass, int64_t cap, unsigned long long* ncls);
__global__ void k_gather_events(PulseDev P, const uint32_t* idx, int64_t n, int blurred, const float* Eb,
                                const float* xb, const float* yb, const float* zb, const int32_t* site,
                                EventRec* out, uint8_t* meta);

// Runs blur .. coincidences on n pulses already in P (device), stream-ordered;
// returns 0 or a GPET_ERR code. Results land in D.single_idx / D.coinc_*,
// counts in cnt. `launches` accumulates the kernel launch count.
int digitize_device(const PulseDev& P, int64_t n, const DigiParams& prm, DigiScratch& D, Counters* cnt,
                    cudaStream_t s, int64_t* launches, int64_t* n_singles_out, int64_t* n_coinc_out);

}  // namespace gpet
