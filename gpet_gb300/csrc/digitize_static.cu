// digitize_static.cu - gpet_digitize_static: the digitizer and coincidence
// sorter with all working memory in one file-scope device array, for callers
// that cannot allocate device memory (see include/gpet.h for who and why).
//
// The array below is the only working memory of this entry point. Host code
// must not pass `g_digi_arena` itself to a kernel: on the host that name is a
// stand-in, not a device address (a kernel given it would fault, or on a
// system where the GPU can reach host memory, silently use the wrong memory).
// Its device address belongs to the CUDA context that loaded the module, not
// to the device number, so every call looks it up again with
// cudaGetSymbolAddress in the context current at that moment (after a
// cudaDeviceReset, or under a non-primary context, a cached address would be
// stale).
#include <cstdio>
#include <cstring>

#include "kernels.h"
#include "../../include/gpet.h"

namespace gpet {

static __device__ __align__(256) unsigned char g_digi_arena[GPET_STATIC_ARENA_BYTES];

namespace {

// device address of g_digi_arena in the current context (looked up on every call)
cudaError_t arena_for_current_context(unsigned char** out)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_digi_arena);
    if (e != cudaSuccess) return e;
    *out = static_cast<unsigned char*>(p);
    return cudaSuccess;
}

// word of DigiScratch::dcount that k_events_to_soa sets when a slot is >= 128
constexpr int kBadSlotWord = 12;

// bump allocator over the arena, 256-byte aligned pieces
struct Carve {
    unsigned char* base;
    size_t off, cap;
    template <class T> T* take(size_t count)
    {
        size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
        if (off + bytes > cap) return nullptr;
        T* p = reinterpret_cast<T*>(base + off);
        off += bytes;
        return p;
    }
};

// slots of 128 or more cannot be packed beside the scatter flag: they are
// counted in *bad_slot and the call is refused, as gpet_digitize refuses them
__global__ void k_events_to_soa(const EventRec* __restrict__ ev, const uint8_t* __restrict__ scat,
                                const uint8_t* __restrict__ slot, int64_t n, PulseDev P,
                                unsigned long long* bad_slot)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const EventRec e = ev[i];
        const uint8_t sl = slot[i];
        if (sl > 0x7fu) atomicAdd(bad_slot, 1ull);
        P.parn[i] = e.parn; P.pann[i] = e.pann; P.modn[i] = e.modn; P.cryn[i] = e.cryn;
        P.siten[i] = e.siten; P.eventid[i] = e.eventid; P.t[i] = e.t;
        P.E[i] = e.E; P.x[i] = e.x; P.y[i] = e.y; P.z[i] = e.z;
        P.meta[i] = (uint8_t)((sl & 0x7fu) | (scat[i] ? 0x80u : 0u));
    }
}

__global__ void k_meta_to_scat(const uint8_t* __restrict__ meta, int64_t n, uint8_t* scat)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        scat[i] = (meta[i] & 0x80u) ? 1 : 0;
}

unsigned grid256(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 152 * 64 ? 152 * 64 : b));
}

void scan(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* aux, uint32_t* total, cudaStream_t s)
{
    int64_t nb = (n + kDigiTile - 1) / kDigiTile;
    if (nb == 0) {
        cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
        return;
    }
    k_scan_reduce<<<(unsigned)nb, 256, 0, s>>>(in, n, aux);
    k_scan_aux<<<1, 1024, 0, s>>>(aux, nb, total);
    k_scan_down<<<(unsigned)nb, 1024, 0, s>>>(in, n, aux, out);
}

void sort(uint64_t*& ka, uint32_t*& va, uint64_t*& kb, uint32_t*& vb, int64_t n, int nbits, uint32_t* hist,
          uint32_t* aux, uint32_t* total, cudaStream_t s)
{
    int64_t launches = 0;
    radix_sort(ka, va, kb, vb, n, nbits, hist, aux, total, s, &launches);
}

int set_err(char* err, int32_t len, int code, const char* msg)
{
    if (err && len > 0) std::snprintf(err, (size_t)len, "%s", msg);
    return code;
}

}  // namespace
}  // namespace gpet

using namespace gpet;

extern "C" int gpet_digitize_static(const gpet_digi_params* prm, const gpet_event* d_pulses, const uint8_t* d_scat,
                                    const uint8_t* d_slot, int64_t n, gpet_event* d_singles, uint8_t* d_single_scat,
                                    int64_t singles_cap, int64_t* d_pairs, uint8_t* d_class, int64_t pairs_cap,
                                    int64_t counts[8], void* stream, char* err, int32_t err_len)
{
    if (!prm || !counts || n < 0 || (n > 0 && (!d_pulses || !d_scat || !d_slot)) || singles_cap < 0 || pairs_cap < 0)
        return set_err(err, err_len, GPET_ERR_ARG, "null pointer or negative size");
    if (n > GPET_STATIC_MAX_PULSES) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "gpet_digitize_static: %lld pulses exceed the maximum of %d",
                      (long long)n, GPET_STATIC_MAX_PULSES);
        return set_err(err, err_len, GPET_ERR_ARG, msg);
    }
    if (prm->coinc_policy < 0 || prm->coinc_policy > 1)
        return set_err(err, err_len, GPET_ERR_ARG, "coinc_policy must be 0 or 1");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // an error left by the caller's earlier work is reported as such and left pending for the caller
    cudaError_t ce = cudaPeekAtLastError();
    if (ce != cudaSuccess) {
        char msg[200];
        std::snprintf(msg, sizeof(msg), "a CUDA error from earlier work is pending (not cleared): %s",
                      cudaGetErrorString(ce));
        return set_err(err, err_len, GPET_ERR_CUDA, msg);
    }
    unsigned char* arena = nullptr;
    ce = arena_for_current_context(&arena);
    if (ce != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    for (int k = 0; k < 8; ++k) counts[k] = 0;

    // carve the working memory for n pulses
    const int64_t N = n > 0 ? n : 1;
    Carve cv{arena, 0, GPET_STATIC_ARENA_BYTES};
    PulseDev P{};
    int32_t* I = cv.take<int32_t>(6 * (size_t)N);
    P.t = cv.take<double>(N);
    float* F = cv.take<float>(4 * (size_t)N);
    P.meta = cv.take<uint8_t>(N);
    DigiScratch D{};
    D.idx_a = cv.take<uint32_t>(N); D.idx_b = cv.take<uint32_t>(N);
    D.key_a = cv.take<uint64_t>(N); D.key_b = cv.take<uint64_t>(N);
    D.torder = cv.take<uint32_t>(N); D.flags = cv.take<uint32_t>(N); D.site = cv.take<int32_t>(N);
    D.sel = cv.take<uint32_t>(N);
    float* B = cv.take<float>(4 * (size_t)N);
    D.single_idx = cv.take<uint32_t>(N);
    D.wcount = cv.take<uint32_t>(N); D.wend = cv.take<uint32_t>(N);
    const int64_t nb = (N + kDigiTile - 1) / kDigiTile;
    D.hist = cv.take<uint32_t>(256 * (size_t)nb);
    D.scan_aux = cv.take<uint32_t>((256 * (size_t)nb + kDigiTile - 1) / kDigiTile + (size_t)nb + 16);
    uint8_t* meta_out = cv.take<uint8_t>(N);
    D.dcount = cv.take<unsigned long long>(16);
    DigiParams* d_prm = cv.take<DigiParams>(1);
    Counters* d_cnt = cv.take<Counters>(1);
    if (!I || !P.t || !F || !P.meta || !D.idx_a || !D.idx_b || !D.key_a || !D.key_b || !D.torder || !D.flags ||
        !D.site || !D.sel || !B || !D.single_idx || !D.wcount || !D.wend || !D.hist || !D.scan_aux || !meta_out ||
        !D.dcount || !d_prm || !d_cnt)
        return set_err(err, err_len, GPET_ERR_CAPACITY, "static arena too small for this input");
    P.parn = I; P.pann = I + N; P.modn = I + 2 * N; P.cryn = I + 3 * N; P.siten = I + 4 * N; P.eventid = I + 5 * N;
    P.E = F; P.x = F + N; P.y = F + 2 * N; P.z = F + 3 * N;
    D.Eb = B; D.xb = B + N; D.yb = B + 2 * N; D.zb = B + 3 * N;
    P.cap = N;

    DigiParams dp{};
    dp.key0 = (uint32_t)prm->seed;
    dp.key1 = (uint32_t)(prm->seed >> 32) + prm->sim_id;
    dp.blurpolicy = prm->blurpolicy; dp.Eref = prm->Eref; dp.Rref = prm->Rref; dp.Eslope = prm->Eslope;
    dp.Sblur = prm->Sblur; dp.Eth = prm->Eth; dp.dlevel = prm->dlevel; dp.dtype = prm->dtype;
    dp.tau = (double)prm->dtime_us; dp.ewin_lo = prm->ewin_lo; dp.ewin_hi = prm->ewin_hi;
    dp.window = prm->coinc_window_ns * 1e-3; dp.coinc_policy = prm->coinc_policy;
    dp.moduleN = prm->moduleN; dp.crystalN = prm->crystalN;

    // the arena keeps the last call's contents: clear the counters
    cudaMemsetAsync(D.dcount, 0, 16 * sizeof(unsigned long long), s);
    cudaMemsetAsync(D.dcount + 8, 0xFF, sizeof(unsigned long long), s);
    cudaMemsetAsync(d_cnt, 0, sizeof(Counters), s);
    cudaMemcpyAsync(d_prm, &dp, sizeof(DigiParams), cudaMemcpyHostToDevice, s);
    unsigned long long hc[kBadSlotWord + 1] = {0};
    if (n > 0) {
        k_events_to_soa<<<grid256(n), 256, 0, s>>>(reinterpret_cast<const EventRec*>(d_pulses), d_scat, d_slot, n, P,
                                                   D.dcount + kBadSlotWord);
        k_blur_threshold<<<grid256(n), 256, 0, s>>>(P, n, d_prm, D.Eb, D.xb, D.yb, D.zb, D.site, D.sel, D.dcount + 0,
                                                    D.dcount + 8);
    }
    cudaMemcpyAsync(hc, D.dcount, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if ((ce = cudaGetLastError()) != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    if (hc[kBadSlotWord] != 0) {
        char msg[160];
        std::snprintf(msg, sizeof(msg), "gpet_digitize_static: %llu pulses have a readout slot of 128 or more",
                      hc[kBadSlotWord]);
        return set_err(err, err_len, GPET_ERR_ARG, msg);
    }
    const int64_t m = (int64_t)hc[0];
    uint32_t* total = reinterpret_cast<uint32_t*>(D.dcount + 4);
    uint64_t *ka = D.key_a, *kb = D.key_b;
    uint32_t *va = D.idx_a, *vb = D.idx_b;
    if (m > 0) {
        const int tbits = launch_time_keys(D.sel, m, P.t, hc + 8, ka, va, s);
        sort(ka, va, kb, vb, m, tbits, D.hist, D.scan_aux, total, s);
        k_tie_fix<<<grid256(m), 256, 0, s>>>(ka, va, m, P.t, P.parn, P.meta);
        cudaMemcpyAsync(D.torder, va, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s);
        const int site_bits = site_key_bits(hc[10]);
        k_site_keys<<<grid256(m), 256, 0, s>>>(D.torder, m, D.site, nullptr, ka, va);
        sort(ka, va, kb, vb, m, site_bits, D.hist, D.scan_aux, total, s);
        k_deadtime<<<grid256(m), 256, 0, s>>>(va, ka, m, P.t, d_prm, 0, D.flags, d_cnt);
        k_window_pred<<<grid256(m), 256, 0, s>>>(D.torder, m, D.flags, D.Eb, nullptr, d_prm, D.sel, d_cnt);
        scan(D.sel, D.wcount, m, D.scan_aux, reinterpret_cast<uint32_t*>(D.dcount + 2), s);
        k_compact<<<grid256(m), 256, 0, s>>>(D.torder, D.sel, D.wcount, m, D.single_idx);
    }
    cudaMemcpyAsync(hc, D.dcount, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    const int64_t ns = m > 0 ? (int64_t)(hc[2] & 0xffffffffull) : 0;
    counts[0] = m; counts[2] = ns;
    if (ns > singles_cap) return set_err(err, err_len, GPET_ERR_CAPACITY, "more singles than singles_cap");
    if (ns > 0 && (!d_singles || !d_single_scat)) return set_err(err, err_len, GPET_ERR_ARG, "null singles buffer");
    int64_t nc = 0;
    if (ns > 0) {
        k_gather_events<<<grid256(ns), 256, 0, s>>>(P, D.single_idx, ns, 1, D.Eb, D.xb, D.yb, D.zb, D.site,
                                                    reinterpret_cast<EventRec*>(d_singles), meta_out);
        k_meta_to_scat<<<grid256(ns), 256, 0, s>>>(meta_out, ns, d_single_scat);
        cudaMemsetAsync(D.wcount, 0, sizeof(uint32_t) * ns, s);
        cudaMemsetAsync(D.wend, 0, sizeof(uint32_t) * ns, s);
        k_coinc_count<<<grid256(ns), 256, 0, s>>>(D.single_idx, ns, P.t, P.pann, nullptr, d_prm, D.wcount, D.wend,
                                                  d_cnt);
        scan(D.wcount, D.sel, ns, D.scan_aux, total, s);
        uint32_t hn = 0;
        cudaMemcpyAsync(&hn, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if ((ce = cudaStreamSynchronize(s)) != cudaSuccess)
            return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
        nc = hn;
        counts[3] = nc;
        if (nc > pairs_cap) return set_err(err, err_len, GPET_ERR_CAPACITY, "more coincidences than pairs_cap");
        if (nc > 0 && (!d_pairs || !d_class)) return set_err(err, err_len, GPET_ERR_ARG, "null coincidence buffer");
        if (nc > 0)
            k_coinc_write<<<grid256(ns), 256, 0, s>>>(D.single_idx, ns, D.wend, D.sel, P.pann, P.eventid, P.meta,
                                                      nullptr, d_prm, d_pairs, d_class, pairs_cap, d_cnt);
    }
    Counters h{};
    cudaMemcpyAsync(&h, d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    if ((ce = cudaGetLastError()) != cudaSuccess) return set_err(err, err_len, GPET_ERR_CUDA, cudaGetErrorString(ce));
    counts[1] = m > 0 ? (int64_t)h.n_dead : 0;
    counts[4] = (int64_t)h.n_true;
    counts[5] = (int64_t)h.n_scat;
    counts[6] = (int64_t)h.n_rand;
    counts[7] = (int64_t)h.n_mult;
    return GPET_OK;
}
