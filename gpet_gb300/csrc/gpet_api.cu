// gpet_api.cu - host runtime behind the C ABI of include/gpet.h: context,
// options, scene upload, run orchestration (the role of main.cu, init and
// sampleParticle/simulateParticle in gPET.cu), output copy-out and writers.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "kernels.h"
#include "loaders.hpp"
#include "surrogate.h"
#include "../../include/gpet.h"
#include "../../include/gpet_surrogate.h"

using namespace gpet;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
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

// grow-only host array, page-locked when the system grants it (device-to-host
// copies into it then run at the host link's rate and asynchronously), else
// ordinary memory (the copies are then staged by the CUDA driver); resize() leaves
// the contents unset
template <class T>
struct PinnedVec {
    T* p = nullptr;
    size_t n = 0, cap = 0;
    bool pinned = false;
    PinnedVec() = default;
    PinnedVec(const PinnedVec&) = delete;
    PinnedVec& operator=(const PinnedVec&) = delete;
    ~PinnedVec() { release(); }
    void release()
    {
        if (p) {
            if (pinned) cudaFreeHost(p);
            else std::free(p);
        }
        p = nullptr;
        cap = n = 0;
        pinned = false;
    }
    cudaError_t resize(size_t m)
    {
        if (m > cap) {
            release();
            if (cudaHostAlloc(reinterpret_cast<void**>(&p), m * sizeof(T), cudaHostAllocDefault) == cudaSuccess) {
                pinned = true;
            } else {
                cudaGetLastError();   // not sticky; fall back to pageable memory
                p = static_cast<T*>(std::malloc(m * sizeof(T)));
                if (!p) return cudaErrorMemoryAllocation;
            }
            cap = m;
        }
        n = m;
        return cudaSuccess;
    }
    void clear() { n = 0; }
    size_t size() const { return n; }
    bool empty() const { return n == 0; }
    T* data() { return p; }
    const T* data() const { return p; }
    const T& operator[](size_t i) const { return p[i]; }
    const T* begin() const { return p; }
    const T* end() const { return p + n; }
};

}  // namespace

// device work buffers and results of one run; a batch's contexts share the
// leader's Work and read their own simulation's slice of the results
struct Work {
    DevBuf q_f, q_t, q_i;                 // detector queues: two, used by alternate chunks
    DevBuf qb_f, qb_t, qb_i;
    int64_t q_cap = 0;
    DevBuf q2_f, q2_t, q2_i, sidx;        // with a surrogate: the Monte Carlo part of the queue, the surrogate's list
    DevBuf ent;                           // entry records of one chunk
    DevBuf serr;                          // surrogate kernel error flag
    DevBuf pb_f, pb_t, pb_n;              // emitted pairs of one wave
    DevBuf pb_wf, pb_wj;                  // the wave's positron walk list
    int64_t pb_cap = 0;
    DevBuf aux;                           // [0] queue count [1] pulses [2] hits [4] Monte Carlo queue [5] surrogate list
                                          // [6] second queue count [8] detector lanes' next entry
    DevBuf cnt;                           // Counters per simulation
    DevBuf sims, prms, segs;              // batch descriptors
    DevBuf p_int, p_t, p_f, p_meta, p_sim;  // pulses: 6 int32, double, 4 float, byte, simulation
    int64_t p_cap = 0;
    DevBuf h_id, h_f, h_sim;
    int64_t h_cap = 0;
    DevBuf exits, source;                 // per photon slot of a chunk
    DevBuf g_ev, g_meta;                  // gathered Event records for copy-out
    DigiScratch dg{};
    DevBuf dg_idx_a, dg_idx_b, dg_key_a, dg_key_b, dg_torder, dg_flags, dg_site, dg_hist, dg_aux, dg_sel, dg_blur,
        dg_single, dg_wcount, dg_wend, dg_dcount;
    std::vector<cudaEvent_t> tev;         // per-launch timing events
    DevBuf d_waves, d_work;               // wave table and photon counters of one chunk
    Wave* h_waves = nullptr;              // pinned staging of the wave table
    size_t h_waves_cap = 0;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};   // per queue: the chunk's launches, replayed while
    std::vector<unsigned char> gkey[2];              // their arguments stay put
    std::vector<cudaEvent_t> dev;         // per chunk: detector stage start, end, surrogate start, end
    // results
    int nsims = 0;
    int64_t n_pulses = 0, n_hits = 0, n_singles = 0, n_coinc = 0;
    int64_t n_digi = 0;                   // pulses digitized: n_pulses plus background singles
    std::vector<Counters> hcnt;           // per simulation
    std::vector<uint8_t> sim_hits;        // per simulation: hits recorded
    std::vector<int64_t> s_off, c_off;    // first single / coincidence of each simulation
    ~Work()
    {
        for (auto& e : tev) cudaEventDestroy(e);
        for (auto& e : dev) cudaEventDestroy(e);
        for (auto& g : gexec) if (g) cudaGraphExecDestroy(g);
        if (h_waves) cudaFreeHost(h_waves);
        if (dg.coinc_pairs) cudaFree(dg.coinc_pairs);
        if (dg.coinc_class) cudaFree(dg.coinc_class);
    }
};

// device buffers of one kind of result on their way to the caller, and the
// end of the last copy out of them
struct Staged {
    DevBuf a, b;
    cudaEvent_t done = nullptr;
    bool pending = false;
};

struct gpet_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;       // detector stage, overlapping the next chunk's transport
    cudaEvent_t qev[4] = {};              // per queue: transport done [0, 1], detector done [2, 3]
    std::string err;
    // options
    uint64_t seed = 20261203ull;
    uint32_t sim_id = 0;
    int64_t n_decays_opt = -1;
    double coinc_window_ns = 4.0;
    int coinc_policy = 0;
    int record_hits = 1;
    int record_exits = 0;
    int64_t chunk_decays = 1ll << 24;
    int64_t sub_decays = 1ll << 20;       // decays per wave: the pair buffer stays in L2
    int phantom_bps = 0;                  // k_phantom blocks per SM (0: as many as fit)
    int drain_period = 32;                // k_phantom compaction period
    int det_threads = 256, src_threads = 256;
    int use_graphs = 1;
    int autotune = 0;                     // tune the launch shape on the first run
    bool tuned = false;
    int record_entries = 0;               // keep the entry records of the detector stage
    int record_source = 0;                // keep the emitted photons (source phase space)
    float noise_lambda_us = 0.0f;         // background singles: mean gap (us), 0 = none
    float noise_emean = 511000.0f, noise_sigma = 0.0f;
    double noise_interval_us = 1000.0;
    int psf_sphere = 0;                   // phantom phase space projected onto the record sphere
    int voxel_palette = 1;                // 16-bit voxel indices into a (density, material) palette
                                          // when the distinct pairs fit (1), or 8-byte pairs (0)
    bool vox_pal = false;                 // the phantom on the device is in palette form
    gpet_surrogate* sur = nullptr;        // learned detector response (not owned)
    std::string base_dir = ".";
    std::string data_dir;
    // host scene
    Config cfg;
    bool have_cfg = false, have_tables = false, have_phantom = false, have_geo = false, have_source = false;
    Tables tab;
    Geometry geo;
    Sources src;
    float tstart = 0.0f, tend = 1.0f;
    std::vector<double> psf;
    int psf_ptype = 0;
    bool use_psf = false;
    int pdim[3] = {0, 0, 0};
    float poff[3] = {0, 0, 0}, psz[3] = {0, 0, 0};
    float maxden_ph[10] = {0};
    bool wck_ph_valid = false;   // wck_ph is built from the loaded tables and maxden_ph
    std::vector<float> wck_ph, wck_det;
    float wck_e0 = 0, wck_ide = 0;
    std::vector<int64_t> src_first, src_count;
    // device scene
    SimDesc sim{};
    DevBuf d_sim, d_xs4, d_cmpsf, d_rayff, d_wck_ph, d_wck_det, d_vox, d_panels, d_psf;
    DevBuf d_vox16, d_pal;                // palette form: per-voxel index, palette (hash table of pairs)
    DevBuf d_mat_stage, d_den_stage, d_maxden;   // phantom upload
    DevBuf d_prmap, d_prmap2;             // uniform-density map of the positron range (and a pass buffer)
    // results of the last run this context took part in
    std::shared_ptr<Work> work;
    // gpet_get_*_async: results gathered into context-owned device buffers
    // (one group for singles, one for coincidences) on `stream`, copied to the
    // caller on `cstream` while the next run proceeds
    cudaStream_t cstream = nullptr;
    cudaEvent_t cready = nullptr;
    Staged st_singles, st_coinc;
    int res_sim = 0;
    PinnedVec<ExitRec> host_exits;       // every photon slot of the run (record_exits)
    std::vector<EntryRec> host_entries;
    PinnedVec<SrcRec> host_source;       // every photon slot of the run (record_source)
    gpet_run_stats last{};
    bool have_results = false;
    cudaEvent_t ev[8] = {};
};

static int fail(gpet_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

static int cuda_fail(gpet_ctx* c, cudaError_t e, const char* what)
{
    return fail(c, GPET_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                            \
    do {                                                    \
        cudaError_t e__ = (call);                           \
        if (e__ != cudaSuccess) return cuda_fail(c, e__, #call); \
    } while (0)

static std::string resolve(const gpet_ctx* c, const std::string& p)
{
    if (p.empty() || p[0] == '/') return p;
    return c->base_dir + "/" + p;
}

// Uniform-density map of the positron-range closed form (prange_uniform):
// m[v] = the largest R <= kPrMax such that every voxel within Chebyshev
// distance R of v has v's density (the same float bits) and lies in
// [1, n-2] on every axis; -1 where v itself is outside that range. The ball
// of radius R around v is the union of the balls of radius R-1 around v's
// 26 neighbours, so m = 1 + min over the neighbours of m where all 26 have
// v's density and lie in the range, else 0; kPrMax Jacobi passes from
// m = min(m, 1) give min(R, kPrMax) exactly.
__device__ __forceinline__ bool pr_interior(int x, int y, int z, int nx, int ny, int nz)
{
    return x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 && z >= 1 && z <= nz - 2;
}

// one thread per voxel on a (32, 8, 1) block grid over (x, y, z); planes
// beyond the grid's z extent (65535) loop
__global__ void k_prmap_init(const float* __restrict__ den, int nx, int ny, int nz, int8_t* __restrict__ m)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    for (int z = blockIdx.z; z < nz; z += gridDim.z) {
        const int64_t v = (int64_t)x + (int64_t)nx * (y + (int64_t)ny * z);
        int8_t r = -1;
        if (pr_interior(x, y, z, nx, ny, nz)) {
            r = 1;
            const unsigned b = __float_as_uint(den[v]);
            for (int dz = -1; dz <= 1 && r; ++dz)
                for (int dy = -1; dy <= 1 && r; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if (!pr_interior(x + dx, y + dy, z + dz, nx, ny, nz) ||
                            __float_as_uint(den[v + dx + (int64_t)nx * (dy + (int64_t)ny * dz)]) != b) {
                            r = 0;
                            break;
                        }
                    }
        }
        m[v] = r;
    }
}

__global__ void k_prmap_pass(const int8_t* __restrict__ m0, int nx, int ny, int nz, int8_t* __restrict__ m1)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    for (int z = blockIdx.z; z < nz; z += gridDim.z) {
        const int64_t v = (int64_t)x + (int64_t)nx * (y + (int64_t)ny * z);
        int r = m0[v];
        if (r >= 1) {
            // v and all its neighbours are in the range and of one density
            int mn = kPrMax;
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if ((dx | dy | dz) == 0) continue;
                        const int q = __ldg(m0 + v + dx + (int64_t)nx * (dy + (int64_t)ny * dz));
                        mn = q < mn ? q : mn;
                    }
            r = mn + 1 < kPrMax ? mn + 1 : kPrMax;
        }
        m1[v] = (int8_t)r;
    }
}

// pack (density, material) into the phantom's 8-byte voxels and take each
// material's largest density for the majorant (initPhantom, initialize.cu:831-884);
// bad counts voxels whose material index is out of range
__global__ void k_pack_phantom(const int32_t* __restrict__ mat, const float* __restrict__ den, int64_t n, int nmat,
                               uint2* __restrict__ vox, unsigned* maxden_bits, unsigned* bad)
{
    __shared__ unsigned smax[16];
    if (threadIdx.x < 16) smax[threadIdx.x] = 0;
    __syncthreads();
    unsigned nbad = 0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int m = mat[v];
        const float d = den[v];
        if (m < 0 || m >= nmat) {
            nbad++;
            continue;
        }
        // positive floats order like their bit patterns
        if (d > 0.0f) atomicMax(&smax[m], __float_as_uint(d));
        vox[v] = make_uint2(__float_as_uint(d), (unsigned)m);
    }
    if (nbad) atomicAdd(bad, nbad);
    __syncthreads();
    if ((int)threadIdx.x < nmat && threadIdx.x < 16 && smax[threadIdx.x]) atomicMax(&maxden_bits[threadIdx.x], smax[threadIdx.x]);
}

// Palette form of the phantom: each voxel's (density bits, material) pair is
// entered in an open-addressing hash table of kPalSlots 64-bit keys (material
// in the high word, density bits in the low word, so a key read as uint2 is
// the voxel record), and the voxel stores its slot. A slot goes from empty to
// its key once, so a plain (cached) read that sees a key sees the final one;
// one that sees an empty slot goes on to the compare-and-swap. Slot numbers
// depend on insertion order, the values they hold do not. Pairs that find no
// slot within kPalProbes probes are counted in bad[1] (the caller falls back
// to the uint2 form).
constexpr int kPalBits = 16;
constexpr uint32_t kPalSlots = 1u << kPalBits;
constexpr int kPalProbes = 256;
constexpr unsigned long long kPalEmpty = ~0ull;

__global__ void k_pack_palette(const int32_t* __restrict__ mat, const float* __restrict__ den, int64_t n, int nmat,
                               uint16_t* __restrict__ vox16, unsigned long long* keys, unsigned* maxden_bits,
                               unsigned* bad)
{
    __shared__ unsigned smax[16];
    if (threadIdx.x < 16) smax[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned nbad = 0, novf = 0;
    // all lanes of a warp run the same iterations (base is block-uniform)
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = base + threadIdx.x;
        const bool in = v < n;
        const int m = in ? mat[v] : 0;
        const float d = in ? den[v] : 0.0f;
        const bool good = in && m >= 0 && m < nmat;
        if (in && !good) nbad++;
        if (good && d > 0.0f) atomicMax(&smax[m], __float_as_uint(d));
        // one probe per distinct pair of the warp (a phantom has few): the
        // lanes holding the same key share their leader's slot; the table is
        // read through L2, where the insertions of other SMs are visible
        const unsigned long long key = good ? (((unsigned long long)(unsigned)m << 32) | __float_as_uint(d))
                                            : kPalEmpty;
        const unsigned grp = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(grp) - 1;
        int slot = -1;
        if (good && lane == leader) {
            uint32_t h = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - kPalBits));
            for (int p = 0; p < kPalProbes; ++p) {
                const unsigned long long cur = __ldcg(&keys[h]);
                if (cur == key) { slot = (int)h; break; }
                if (cur == kPalEmpty) {
                    const unsigned long long prev = atomicCAS(&keys[h], kPalEmpty, key);
                    if (prev == kPalEmpty || prev == key) { slot = (int)h; break; }
                }
                h = (h + 1) & (kPalSlots - 1);
            }
        }
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (good) {
            if (slot < 0) novf++;
            else vox16[v] = (uint16_t)slot;
        }
    }
    if (nbad) atomicAdd(bad, nbad);
    if (novf) atomicAdd(bad + 1, novf);
    __syncthreads();
    if ((int)threadIdx.x < nmat && threadIdx.x < 16 && smax[threadIdx.x]) atomicMax(&maxden_bits[threadIdx.x], smax[threadIdx.x]);
}

// phantom-scatter flag (0/1) from the pulse meta byte, in place
__global__ void k_scat_flags(uint8_t* meta, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        meta[i] = (meta[i] & 0x80u) ? 1 : 0;
}

// coincidences of one simulation, pairs as indices into its own singles, into
// device or mapped host memory (cls may be null)
__global__ void k_coinc_out(const int64_t* __restrict__ pairs, const uint8_t* __restrict__ klass, int64_t n,
                            int64_t soff, int64_t* dst, uint8_t* cls)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const longlong2 v = reinterpret_cast<const longlong2*>(pairs)[i];
        dst[2 * i] = v.x - soff;
        dst[2 * i + 1] = v.y - soff;
        if (cls) cls[i] = klass[i];
    }
}

extern "C" {

int gpet_create(int device, gpet_ctx** out)
{
    if (!out) return GPET_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return GPET_ERR_NOGPU;
    if (device < 0 || device >= n) return GPET_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return GPET_ERR_CUDA;
    if (transport_kernels_loadable() != cudaSuccess) return GPET_ERR_NOGPU;
    auto* c = new gpet_ctx();
    c->device = device;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return GPET_ERR_CUDA;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    for (auto& e : c->qev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return GPET_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&c->cstream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        cudaStreamDestroy(c->stream2);
        delete c;
        return GPET_ERR_CUDA;
    }
    cudaEventCreateWithFlags(&c->cready, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->st_singles.done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&c->st_coinc.done, cudaEventDisableTiming);
    *out = c;
    return GPET_OK;
}

void gpet_destroy(gpet_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->stream2);
    cudaStreamSynchronize(c->cstream);
    for (auto& e : c->ev) if (e) cudaEventDestroy(e);
    for (auto& e : c->qev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {c->cready, c->st_singles.done, c->st_coinc.done})
        if (e) cudaEventDestroy(e);
    c->work.reset();
    cudaStreamDestroy(c->stream);
    cudaStreamDestroy(c->stream2);
    cudaStreamDestroy(c->cstream);
    delete c;
}

const char* gpet_last_error(gpet_ctx* c)
{
    return c ? c->err.c_str() : "null context";
}

int gpet_set_option(gpet_ctx* c, const char* key, const char* value)
{
    if (!c || !key || !value) return GPET_ERR_ARG;
    std::string k(key), v(value);
    char* end = nullptr;
    if (k == "seed") c->seed = std::strtoull(value, &end, 10);
    else if (k == "sim_id") c->sim_id = (uint32_t)std::strtoul(value, &end, 10);
    else if (k == "n_decays") c->n_decays_opt = std::strtoll(value, &end, 10);
    else if (k == "coinc_window_ns") c->coinc_window_ns = std::strtod(value, &end);
    else if (k == "coinc_policy") c->coinc_policy = (int)std::strtol(value, &end, 10);
    else if (k == "record_hits") c->record_hits = (int)std::strtol(value, &end, 10);
    else if (k == "record_exits") c->record_exits = (int)std::strtol(value, &end, 10);
    else if (k == "chunk_decays") c->chunk_decays = std::strtoll(value, &end, 10);
    else if (k == "sub_decays") c->sub_decays = std::strtoll(value, &end, 10);
    else if (k == "phantom_blocks_per_sm") c->phantom_bps = (int)std::strtol(value, &end, 10);
    else if (k == "drain_period") c->drain_period = (int)std::strtol(value, &end, 10);
    else if (k == "detector_threads") c->det_threads = (int)std::strtol(value, &end, 10);
    else if (k == "source_threads") c->src_threads = (int)std::strtol(value, &end, 10);
    else if (k == "use_graphs") c->use_graphs = (int)std::strtol(value, &end, 10);
    else if (k == "autotune") c->autotune = (int)std::strtol(value, &end, 10);
    else if (k == "record_entries") c->record_entries = (int)std::strtol(value, &end, 10);
    else if (k == "record_source") c->record_source = (int)std::strtol(value, &end, 10);
    else if (k == "psf_sphere") c->psf_sphere = (int)std::strtol(value, &end, 10);
    else if (k == "voxel_palette") c->voxel_palette = (int)std::strtol(value, &end, 10);
    else if (k == "noise_lambda_us") c->noise_lambda_us = std::strtof(value, &end);
    else if (k == "noise_emean_ev") c->noise_emean = std::strtof(value, &end);
    else if (k == "noise_sigma_ev") c->noise_sigma = std::strtof(value, &end);
    else if (k == "noise_interval_us") c->noise_interval_us = std::strtod(value, &end);
    else if (k == "base_dir") { c->base_dir = v; return GPET_OK; }
    else if (k == "data_dir") { c->data_dir = v; return GPET_OK; }
    else return fail(c, GPET_ERR_ARG, "unknown option " + k);
    if (end == value || (end && *end)) return fail(c, GPET_ERR_ARG, "bad value for " + k + ": " + v);
    if (c->coinc_policy < 0 || c->coinc_policy > 1) return fail(c, GPET_ERR_ARG, "coinc_policy must be 0 or 1");
    if (c->chunk_decays < 1024) return fail(c, GPET_ERR_ARG, "chunk_decays must be >= 1024");
    if (c->sub_decays < 1024 || c->sub_decays > (1ll << 28))
        return fail(c, GPET_ERR_ARG, "sub_decays must be 1024 .. 2^28");
    if (c->phantom_bps < 0 || c->phantom_bps > 32) return fail(c, GPET_ERR_ARG, "phantom_blocks_per_sm must be 0..32");
    if (!(c->noise_lambda_us >= 0.0f) || !(c->noise_interval_us > 0.0) || !(c->noise_sigma >= 0.0f))
        return fail(c, GPET_ERR_ARG, "noise_lambda_us >= 0, noise_interval_us > 0, noise_sigma_ev >= 0");
    if (c->noise_lambda_us > 0.0f && c->noise_interval_us > 1024.0 * c->noise_lambda_us)
        return fail(c, GPET_ERR_ARG, "noise_interval_us may hold at most 1024 mean gaps");
    if (c->drain_period < 1 || c->drain_period > 32) return fail(c, GPET_ERR_ARG, "drain_period must be 1..32");
    if (c->voxel_palette < 0 || c->voxel_palette > 1) return fail(c, GPET_ERR_ARG, "voxel_palette must be 0 or 1");
    for (int t : {c->det_threads, c->src_threads})
        if (t < 32 || t > 256 || t % 32) return fail(c, GPET_ERR_ARG, "threads per block must be 32..256, a multiple of 32");
    return GPET_OK;
}

// ---------------------------------------------------------------- tables
static double lerp_d(const Tables& t, const float* tab, double e, float idle)
{
    double x = (double)idle * (e - (double)t.energy[0]);
    if (!(x > 0.0)) return tab[0];
    if (x >= t.ne - 1) return tab[t.ne - 1];
    int i = (int)x;
    double f = x - i;
    return tab[i] + f * ((double)tab[i + 1] - (double)tab[i]);
}

// Woodcock majorant (replaces iniwck, initialize.cu:773-829, 919-966): node i
// holds 1/max_m rho_max(m) max(mu_m over [e_{i-1}, e_{i+1}]) of the linearly
// interpolated tables, so the interpolated majorant bounds every material.
static void build_wck(const Tables& t, float idle, const float* maxden, std::vector<float>& w, float& e0, float& ide)
{
    float de = (t.emax - t.eminph) / (float)kNwck;
    e0 = t.eminph;
    ide = 1.0f / de;
    w.assign(kNwck, 0.0f);
    for (int i = 0; i < kNwck; ++i) {
        double lo = (double)t.eminph + (double)de * (double)(i > 0 ? i - 1 : 0);
        double hi = (double)t.eminph + (double)de * (double)(i + 1);
        double best = 0.0;
        for (int m = 0; m < t.nmat; ++m) {
            if (!(maxden[m] > 0.0f)) continue;
            const float* tb = &t.lamph[(size_t)m * t.ne];
            double mx = lerp_d(t, tb, lo, idle);
            double v = lerp_d(t, tb, hi, idle);
            if (v > mx) mx = v;
            double xlo = (double)idle * (lo - (double)t.energy[0]);
            double xhi = (double)idle * (hi - (double)t.energy[0]);
            int k0 = (int)std::ceil(xlo), k1 = (int)std::floor(xhi);
            if (k0 < 0) k0 = 0;
            if (k1 > t.ne - 1) k1 = t.ne - 1;
            for (int k = k0; k <= k1; ++k)
                if (tb[k] > mx) mx = tb[k];
            mx *= (double)maxden[m];
            if (mx > best) best = mx;
        }
        w[i] = (float)(1.0 / best);
    }
}

static float table_idle(const Tables& t) { return (float)(t.ne - 1) / (t.energy[t.ne - 1] - t.energy[0]); }

int gpet_load_tables(gpet_ctx* c, const char* data_dir)
{
    if (!c || !data_dir) return GPET_ERR_ARG;
    cudaSetDevice(c->device);
    Tables t;
    std::string e = read_tables(data_dir, t);
    if (!e.empty()) return fail(c, GPET_ERR_IO, e);
    c->tab = std::move(t);
    const Tables& T = c->tab;
    std::vector<float4> xs((size_t)T.nmat * T.ne);
    for (int m = 0; m < T.nmat; ++m)
        for (int i = 0; i < T.ne; ++i) {
            size_t k = (size_t)m * T.ne + i;
            xs[k] = make_float4(T.lamph[k], T.compt[k], T.rayle[k], T.phote[k]);
        }
    CK(c->d_xs4.ensure(xs.size() * sizeof(float4)));
    CK(cudaMemcpy(c->d_xs4.p, xs.data(), xs.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(c->d_cmpsf.ensure(T.cmpsf.size() * 4));
    CK(cudaMemcpy(c->d_cmpsf.p, T.cmpsf.data(), T.cmpsf.size() * 4, cudaMemcpyHostToDevice));
    CK(c->d_rayff.ensure(T.rayff.size() * 4));
    CK(cudaMemcpy(c->d_rayff.p, T.rayff.data(), T.rayff.size() * 4, cudaMemcpyHostToDevice));
    c->have_tables = true;
    c->wck_ph_valid = false;
    return GPET_OK;
}

int gpet_set_phantom(gpet_ctx* c, const int32_t* mat, const float* den, const int32_t dims[3], const float offset[3],
                     const float size[3])
{
    if (!c || !mat || !den || !dims || !offset || !size) return GPET_ERR_ARG;
    if (!c->have_tables) return fail(c, GPET_ERR_ARG, "load the tables before the phantom");
    if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(c, GPET_ERR_ARG, "phantom dimensions must be >= 1");
    if ((int64_t)dims[0] * dims[1] * dims[2] > INT32_MAX)
        return fail(c, GPET_ERR_ARG, "a phantom holds at most 2^31 - 1 voxels");
    CK(cudaSetDevice(c->device));
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    // the caller's arrays go to the device as they are (a DMA when the caller's
    // memory is pinned) and are packed and checked there
    c->have_phantom = false;
    CK(c->d_mat_stage.ensure((size_t)n * 4));
    CK(c->d_den_stage.ensure((size_t)n * 4));
    CK(c->d_maxden.ensure(32 * 4));
    CK(cudaMemsetAsync(c->d_maxden.p, 0, 32 * 4, c->stream));
    CK(cudaMemcpyAsync(c->d_mat_stage.p, mat, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_den_stage.p, den, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
    unsigned h[18] = {0};
    // palette form (2 B per voxel: a 256 x 256 x 512 phantom stays in L2)
    // unless switched off or the distinct pairs do not fit
    bool pal = c->voxel_palette == 1;
    if (pal) {
        CK(c->d_vox16.ensure((size_t)n * 2));
        CK(c->d_pal.ensure((size_t)kPalSlots * 8));
        CK(cudaMemsetAsync(c->d_pal.p, 0xFF, (size_t)kPalSlots * 8, c->stream));
        k_pack_palette<<<(unsigned)blocks, 256, 0, c->stream>>>(
            c->d_mat_stage.as<int32_t>(), c->d_den_stage.as<float>(), n, c->tab.nmat, c->d_vox16.as<uint16_t>(),
            c->d_pal.as<unsigned long long>(), c->d_maxden.as<unsigned>(), c->d_maxden.as<unsigned>() + 16);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h, c->d_maxden.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (h[17]) {   // too many distinct pairs: the uint2 form
            pal = false;
            CK(cudaMemsetAsync(c->d_maxden.p, 0, 32 * 4, c->stream));
        }
    }
    if (!pal) {
        CK(c->d_vox.ensure((size_t)n * sizeof(uint2)));
        k_pack_phantom<<<(unsigned)blocks, 256, 0, c->stream>>>(c->d_mat_stage.as<int32_t>(),
                                                                 c->d_den_stage.as<float>(), n, c->tab.nmat,
                                                                 c->d_vox.as<uint2>(), c->d_maxden.as<unsigned>(),
                                                                 c->d_maxden.as<unsigned>() + 16);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h, c->d_maxden.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->vox_pal = pal;
    if (h[16]) return fail(c, GPET_ERR_ARG, "phantom material index out of range");
    {
        CK(c->d_prmap.ensure((size_t)n));
        CK(c->d_prmap2.ensure((size_t)n));
        int8_t* m[2] = {c->d_prmap.as<int8_t>(), c->d_prmap2.as<int8_t>()};
        // kPrMax - 1 passes after the first: the last one lands in d_prmap
        int cur = (kPrMax - 1) % 2;
        const dim3 pb(32, 8, 1), pg((dims[0] + 31) / 32, (dims[1] + 7) / 8, std::min(dims[2], 65535));
        k_prmap_init<<<pg, pb, 0, c->stream>>>(c->d_den_stage.as<float>(), dims[0], dims[1], dims[2], m[cur]);
        CK(cudaGetLastError());
        for (int p = 1; p < kPrMax; ++p) {
            k_prmap_pass<<<pg, pb, 0, c->stream>>>(m[cur], dims[0], dims[1], dims[2], m[cur ^ 1]);
            CK(cudaGetLastError());
            cur ^= 1;
        }
    }
    float maxden[10] = {0};
    for (int m = 0; m < 10 && m < c->tab.nmat; ++m) std::memcpy(&maxden[m], &h[m], 4);
    for (int k = 0; k < 3; ++k) { c->pdim[k] = dims[k]; c->poff[k] = offset[k]; c->psz[k] = size[k]; }
    // the majorant depends on the tables and the densest voxel of each
    // material only: a phantom with the same maxima keeps it
    if (!c->wck_ph_valid || std::memcmp(c->maxden_ph, maxden, sizeof(maxden)) != 0) {
        c->wck_ph_valid = false;
        std::memcpy(c->maxden_ph, maxden, sizeof(maxden));
        build_wck(c->tab, table_idle(c->tab), maxden, c->wck_ph, c->wck_e0, c->wck_ide);
        CK(c->d_wck_ph.ensure(kNwck * 4));
        CK(cudaMemcpy(c->d_wck_ph.p, c->wck_ph.data(), kNwck * 4, cudaMemcpyHostToDevice));
        c->wck_ph_valid = true;
    }
    c->have_phantom = true;
    return GPET_OK;
}

int gpet_load_geometry(gpet_ctx* c, const char* path)
{
    if (!c || !path) return GPET_ERR_ARG;
    if (!c->have_tables) return fail(c, GPET_ERR_ARG, "load the tables before the geometry");
    cudaSetDevice(c->device);
    Geometry g;
    std::string e = read_geometry(path, g);
    if (!e.empty()) return fail(c, GPET_ERR_IO, e);
    for (int k = 0; k < 2; ++k)
        if (g.det_mat[k] < 0 || g.det_mat[k] >= c->tab.nmat) return fail(c, GPET_ERR_ARG, "detector material out of range");
    for (int k = 2; k < g.ndetmat; ++k)
        if (g.det_mat[k] < 0 || g.det_mat[k] >= c->tab.nmat) return fail(c, GPET_ERR_ARG, "detector material out of range");
    c->geo = std::move(g);
    float dmax[10] = {0};
    for (int k = 0; k < 2; ++k)
        if (c->geo.det_den[k] > dmax[c->geo.det_mat[k]]) dmax[c->geo.det_mat[k]] = c->geo.det_den[k];
    for (int k = 2; k < c->geo.ndetmat; ++k)
        if (c->geo.det_den[k] > dmax[c->geo.det_mat[k]]) dmax[c->geo.det_mat[k]] = c->geo.det_den[k];
    float e0, ide;
    build_wck(c->tab, table_idle(c->tab), dmax, c->wck_det, e0, ide);
    CK(c->d_wck_det.ensure(kNwck * 4));
    CK(cudaMemcpy(c->d_wck_det.p, c->wck_det.data(), kNwck * 4, cudaMemcpyHostToDevice));
    CK(c->d_panels.ensure(c->geo.panels.size() * 4));
    CK(cudaMemcpy(c->d_panels.p, c->geo.panels.data(), c->geo.panels.size() * 4, cudaMemcpyHostToDevice));
    c->have_geo = true;
    return GPET_OK;
}

int gpet_set_source_file(gpet_ctx* c, const char* path, float tstart, float tend)
{
    if (!c || !path) return GPET_ERR_ARG;
    Sources s;
    std::string e = read_sources(path, s);
    if (!e.empty()) return fail(c, GPET_ERR_IO, e);
    if ((int)s.natom.size() > kMaxSrc) return fail(c, GPET_ERR_ARG, "at most 64 sources");
    for (auto t : s.type)
        if (t < 0 || t >= (int)c->tab.iso_halftime.size()) return fail(c, GPET_ERR_ARG, "isotope type out of range");
    c->src = std::move(s);
    c->tstart = tstart;
    c->tend = tend;
    c->use_psf = false;
    c->have_source = true;
    return GPET_OK;
}

int gpet_set_source_psf(gpet_ctx* c, const double* rec8, int64_t n, int ptype)
{
    if (!c || (!rec8 && n > 0) || n < 0 || (ptype != 0 && ptype != 1)) return GPET_ERR_ARG;
    c->psf.assign(rec8, rec8 + 8 * n);
    c->psf_ptype = ptype;
    c->use_psf = true;
    c->have_source = true;
    return GPET_OK;
}

int gpet_load_config(gpet_ctx* c, const char* path)
{
    if (!c || !path) return GPET_ERR_ARG;
    Config cfg;
    std::string e = read_config(path, cfg);
    if (!e.empty()) return fail(c, GPET_ERR_IO, e);
    c->cfg = cfg;
    c->have_cfg = true;
    std::string dd = c->data_dir.empty() ? c->base_dir + "/data" : c->data_dir;
    int rc = gpet_load_tables(c, dd.c_str());
    if (rc) return rc;
    const int64_t n = (int64_t)cfg.pdim[0] * cfg.pdim[1] * cfg.pdim[2];
    if (n <= 0) return fail(c, GPET_ERR_IO, "phantom dimension must be positive");
    std::vector<int32_t> mat;
    std::vector<float> den;
    e = read_phantom(resolve(c, cfg.matfile), resolve(c, cfg.denfile), n, mat, den);
    if (!e.empty()) return fail(c, GPET_ERR_IO, e);
    rc = gpet_set_phantom(c, mat.data(), den.data(), cfg.pdim, cfg.poffset, cfg.psize);
    if (rc) return rc;
    rc = gpet_load_geometry(c, resolve(c, cfg.geofile).c_str());
    if (rc) return rc;
    if (cfg.usepsf) {
        std::vector<double> rec;
        e = read_psf(resolve(c, cfg.sourcefile), cfg.nparticle, rec);
        if (!e.empty()) return fail(c, GPET_ERR_IO, e);
        return gpet_set_source_psf(c, rec.data(), (int64_t)rec.size() / 8, cfg.ptype);
    }
    return gpet_set_source_file(c, resolve(c, cfg.sourcefile).c_str(), cfg.tstart, cfg.tend);
}

// ---------------------------------------------------------------- run
// decays per source (gPET.cu:204-208, 264-272: floor(N_t (1 - 2^(-dt/T)))
// with N_t = floor(natom 2^(-tstart/T))); an exact total is split over the
// sources in proportion (largest remainder).
static std::string source_layout(gpet_ctx* c)
{
    const Sources& s = c->src;
    const double dt = (double)(c->tend - c->tstart);
    std::vector<int64_t> ex(s.natom.size());
    double tot = 0;
    for (size_t i = 0; i < s.natom.size(); ++i) {
        double th = (double)c->tab.iso_halftime[s.type[i]];
        double nt = std::floor((double)s.natom[i] * std::pow(2.0, -(double)c->tstart / th));
        ex[i] = (int64_t)std::floor(nt * (1.0 - std::pow(2.0, -dt / th)));
        tot += (double)ex[i];
    }
    std::vector<int64_t> cnt = ex;
    if (c->n_decays_opt >= 0) {
        if (!(tot > 0)) return "no source decays in the acquisition window";
        std::vector<double> quota(ex.size());
        int64_t sum = 0;
        for (size_t i = 0; i < ex.size(); ++i) {
            quota[i] = (double)c->n_decays_opt * (double)ex[i] / tot;
            cnt[i] = (int64_t)std::floor(quota[i]);
            sum += cnt[i];
        }
        std::vector<size_t> order(ex.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return (quota[a] - (double)cnt[a]) > (quota[b] - (double)cnt[b]);
        });
        for (int64_t r = 0; r < c->n_decays_opt - sum; ++r) cnt[order[(size_t)r]]++;
    }
    c->src_first.assign(cnt.size(), 0);
    c->src_count = cnt;
    for (size_t i = 1; i < cnt.size(); ++i) c->src_first[i] = c->src_first[i - 1] + cnt[i - 1];
    return "";
}

// the bound of the panel entry faces used by may_reach_panels: every face
// must be parallel to the z axis; its plane's distance to the axis bounds the
// face from below, its corners bound its z range; both padded
static void ring_bound(const Geometry& g, SimDesc& S)
{
    S.ring_test = 0;
    double zmin = 1e30, zmax = -1e30, rin = 1e30;
    // whether every face takes only photons moving toward it from the axis
    // side: enter_panel's direction test (u . n) * dir_x >= 0 with the sign of
    // dir_x equal to that of n . o (the plane's side as seen from the axis)
    bool toward = true;
    for (int i = 0; i < g.npanels; ++i) {
        const float* P = &g.panels[(size_t)i * kPanelStride];
        const double nx = P[21], ny = P[22], nz = P[23];
        const double nxy = std::sqrt(nx * nx + ny * ny);
        if (std::fabs(nz) > 1e-6 || !(nxy > 0.5)) return;
        const double d = std::fabs(nx * P[15] + ny * P[16]) / nxy;
        rin = std::min(rin, d);
        const double no = nx * P[15] + ny * P[16] + nz * P[17];
        if (!(P[18] != 0.0f) || !(no != 0.0) || (P[18] > 0.0f) != (no > 0.0)) toward = false;
        for (int sy = -1; sy <= 1; sy += 2)
            for (int sz = -1; sz <= 1; sz += 2) {
                const double z = (double)P[17] + sy * 0.5 * P[1] * P[26] + sz * 0.5 * P[2] * P[29];
                zmin = std::min(zmin, z);
                zmax = std::max(zmax, z);
            }
    }
    const double pad = 1e-3;
    const double r = rin * (1.0 - 1e-4) - pad;
    if (!(r > 0.0) || !(zmax >= zmin)) return;
    S.ring_zmin = (float)(zmin - pad - 1e-4 * std::fabs(zmin));
    S.ring_zmax = (float)(zmax + pad + 1e-4 * std::fabs(zmax));
    S.ring_rin2 = (float)(r * r);
    S.ring_test = toward ? 2 : 1;
}

static int build_sim(gpet_ctx* c)
{
    SimDesc& S = c->sim;
    std::memset(&S, 0, sizeof(S));
    S.key0 = (uint32_t)c->seed;
    S.key1 = (uint32_t)(c->seed >> 32) + c->sim_id;
    const Tables& T = c->tab;
    S.nmat = T.nmat; S.ne = T.ne; S.e0 = T.energy[0]; S.idle = table_idle(T);
    S.xs4 = c->d_xs4.as<float4>();
    S.ncp_c = T.ncp_c; S.ne_c = T.ne_c; S.idcp_c = 1.0f / T.dcp_c; S.ide_c = 1.0f / T.de_c;
    S.cmpsf = c->d_cmpsf.as<float>();
    S.ncp_r = T.ncp_r; S.ne_r = T.ne_r; S.idcp_r = 1.0f / T.dcp_r; S.ide_r = 1.0f / T.de_r;
    S.rayff = c->d_rayff.as<float>();
    S.wck_e0 = c->wck_e0; S.wck_ide = c->wck_ide;
    S.wck_ph = c->d_wck_ph.as<float>(); S.wck_det = c->d_wck_det.as<float>();
    S.nx = c->pdim[0]; S.ny = c->pdim[1]; S.nz = c->pdim[2];
    S.dx = c->psz[0] / (float)c->pdim[0]; S.dy = c->psz[1] / (float)c->pdim[1]; S.dz = c->psz[2] / (float)c->pdim[2];
    S.idx = 1.0f / S.dx; S.idy = 1.0f / S.dy; S.idz = 1.0f / S.dz;
    S.offx = c->poff[0]; S.offy = c->poff[1]; S.offz = c->poff[2];
    S.vox = c->vox_pal ? c->d_pal.as<uint2>() : c->d_vox.as<uint2>();
    S.vox16 = c->vox_pal ? c->d_vox16.as<uint16_t>() : nullptr;
    S.prmap = c->d_prmap.as<int8_t>();
    // the uploaded density array (still on the device) serves the positron
    // range's lookups while it fits comfortably in L2; larger phantoms use
    // the 16-bit palette records, which stay in L2 longer
    const int64_t nvox = (int64_t)c->pdim[0] * c->pdim[1] * c->pdim[2];
    S.den = nvox * 4 <= ((int64_t)64 << 20) ? c->d_den_stage.as<float>() : nullptr;
    S.prdmin = std::fmin(S.dx, std::fmin(S.dy, S.dz));
    S.npanels = c->geo.npanels;
    S.panels = c->d_panels.as<float>();
    S.ndetmat = c->geo.ndetmat;
    for (int k = 0; k < c->geo.ndetmat; ++k) { S.det_mat[k] = c->geo.det_mat[k]; S.det_den[k] = c->geo.det_den[k]; }
    S.moduleN = c->geo.moduleN; S.crystalN = c->geo.crystalN; S.moduleNy = c->geo.moduleNy; S.crystalNy = c->geo.crystalNy;
    const Config& cf = c->cfg;
    S.nsurface = c->have_cfg ? (int)cf.surfaces.size() / 10 : 0;
    for (int k = 0; k < 10 * S.nsurface; ++k) S.surface[k] = cf.surfaces[k];
    S.noncol_sigma = c->have_cfg ? cf.noncol_sigma : 0.0037056f;
    S.eabsph = c->have_cfg ? cf.eabsph : 1000.0f;
    S.useprange = c->have_cfg ? cf.useprange : 0;
    S.rdepth = c->have_cfg ? cf.rdepth : 2;
    ring_bound(c->geo, S);
    S.rpolicy = c->have_cfg ? cf.rpolicy : 1;
    if (c->use_psf) {
        S.npsf = (int64_t)c->psf.size() / 8;
        S.psf_ptype = c->psf_ptype;
        if (cudaSuccess != c->d_psf.ensure(c->psf.size() * 8)) return fail(c, GPET_ERR_CUDA, "psf upload");
        cudaMemcpy(c->d_psf.p, c->psf.data(), c->psf.size() * 8, cudaMemcpyHostToDevice);
        S.psf = c->d_psf.as<double>();
        S.nsrc = 0;
    } else {
        std::string e = source_layout(c);
        if (!e.empty()) return fail(c, GPET_ERR_ARG, e);
        S.nsrc = (int)c->src.natom.size();
        const double dt = (double)(c->tend - c->tstart);
        for (int i = 0; i < S.nsrc; ++i) {
            int ty = c->src.type[i];
            S.src_end[i] = c->src_first[i] + c->src_count[i];
            S.src_type[i] = ty;
            S.src_shape[i] = c->src.shape[i];
            for (int k = 0; k < 6; ++k) S.src_coef[i][k] = c->src.coef[6 * i + k];
            double th = (double)c->tab.iso_halftime[ty];
            double tau = th / 0.69314718055994530942;
            S.src_ntau_us[i] = -tau * 1e6;
            S.src_cfac[i] = -std::expm1(-dt / tau);
            S.iso_ratio[i] = c->tab.iso_ratio[ty];
            for (int k = 0; k < 8; ++k) S.iso_coef[i][k] = c->tab.iso_coef[8 * ty + k];
        }
        S.tstart_us = (double)c->tstart * 1e6;
    }
    if (cudaSuccess != c->d_sim.ensure(sizeof(SimDesc))) return fail(c, GPET_ERR_CUDA, "sim upload");
    cudaMemcpyAsync(c->d_sim.p, &S, sizeof(SimDesc), cudaMemcpyHostToDevice, c->stream);
    return GPET_OK;
}

static int64_t total_decays(const gpet_ctx* c)
{
    if (c->use_psf) return (int64_t)c->psf.size() / 8;
    int64_t t = 0;
    for (auto v : c->src_count) t += v;
    return t;
}

}  // extern "C"

// ---------------------------------------------------------------- run
// grow a structure-of-arrays pulse buffer, keeping the first `used` entries
static int grow_pulses(gpet_ctx* c, Work& W, int64_t need, int64_t used)
{
    if (need <= W.p_cap) return GPET_OK;
    int64_t cap = std::max<int64_t>(need + need / 2, 1 << 20);
    DevBuf ni, nt, nf, nm, ns;
    CK(ni.ensure((size_t)cap * 6 * 4));
    CK(nt.ensure((size_t)cap * 8));
    CK(nf.ensure((size_t)cap * 4 * 4));
    CK(nm.ensure((size_t)cap));
    CK(ns.ensure((size_t)cap * 4));
    if (used > 0) {
        for (int a = 0; a < 6; ++a)
            CK(cudaMemcpyAsync(ni.as<int32_t>() + a * cap, W.p_int.as<int32_t>() + a * W.p_cap, used * 4,
                               cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(nt.p, W.p_t.p, used * 8, cudaMemcpyDeviceToDevice, c->stream));
        for (int a = 0; a < 4; ++a)
            CK(cudaMemcpyAsync(nf.as<float>() + a * cap, W.p_f.as<float>() + a * W.p_cap, used * 4,
                               cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(nm.p, W.p_meta.p, used, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(ns.p, W.p_sim.p, used * 4, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    std::swap(W.p_int.p, ni.p); std::swap(W.p_int.bytes, ni.bytes);
    std::swap(W.p_t.p, nt.p); std::swap(W.p_t.bytes, nt.bytes);
    std::swap(W.p_f.p, nf.p); std::swap(W.p_f.bytes, nf.bytes);
    std::swap(W.p_meta.p, nm.p); std::swap(W.p_meta.bytes, nm.bytes);
    std::swap(W.p_sim.p, ns.p); std::swap(W.p_sim.bytes, ns.bytes);
    W.p_cap = cap;
    return GPET_OK;
}

static int grow_hits(gpet_ctx* c, Work& W, int64_t need, int64_t used)
{
    if (need <= W.h_cap) return GPET_OK;
    int64_t cap = std::max<int64_t>(need + need / 2, 1 << 20);
    DevBuf ni, nf, ns;
    CK(ni.ensure((size_t)cap * 20));
    CK(nf.ensure((size_t)cap * 20));
    CK(ns.ensure((size_t)cap * 4));
    if (used > 0) {
        CK(cudaMemcpyAsync(ni.p, W.h_id.p, used * 20, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(nf.p, W.h_f.p, used * 20, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(ns.p, W.h_sim.p, used * 4, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    std::swap(W.h_id.p, ni.p); std::swap(W.h_id.bytes, ni.bytes);
    std::swap(W.h_f.p, nf.p); std::swap(W.h_f.bytes, nf.bytes);
    std::swap(W.h_sim.p, ns.p); std::swap(W.h_sim.bytes, ns.bytes);
    W.h_cap = cap;
    return GPET_OK;
}

static PulseDev pulse_view(Work& W)
{
    PulseDev P;
    int32_t* I = W.p_int.as<int32_t>();
    float* F = W.p_f.as<float>();
    int64_t cap = W.p_cap;
    P.parn = I; P.pann = I + cap; P.modn = I + 2 * cap; P.cryn = I + 3 * cap; P.siten = I + 4 * cap;
    P.eventid = I + 5 * cap;
    P.t = W.p_t.as<double>();
    P.E = F; P.x = F + cap; P.y = F + 2 * cap; P.z = F + 3 * cap;
    P.meta = W.p_meta.as<uint8_t>();
    P.sim = W.nsims > 1 ? W.p_sim.as<int32_t>() : nullptr;
    P.count = W.aux.as<unsigned long long>() + 1;
    P.cap = cap;
    return P;
}

static int ensure_digi(gpet_ctx* c, Work& W, int64_t n)
{
    int64_t cap = std::max<int64_t>(n, 1024);
    if (cap > W.dg.cap) {
        cap = cap + cap / 4;
        CK(W.dg_idx_a.ensure(cap * 4)); CK(W.dg_idx_b.ensure(cap * 4));
        CK(W.dg_key_a.ensure(cap * 8)); CK(W.dg_key_b.ensure(cap * 8));
        CK(W.dg_torder.ensure(cap * 4)); CK(W.dg_flags.ensure(cap * 4)); CK(W.dg_site.ensure(cap * 4));
        CK(W.dg_sel.ensure(cap * 4)); CK(W.dg_blur.ensure(cap * 16)); CK(W.dg_single.ensure(cap * 4));
        CK(W.dg_wcount.ensure(cap * 4)); CK(W.dg_wend.ensure(cap * 4));
        int64_t nb = (cap + 4095) / 4096;
        CK(W.dg_hist.ensure((size_t)256 * nb * 4));
        int64_t na = (256 * nb + 4095) / 4096 + (cap + 4095) / 4096 + 16;
        CK(W.dg_aux.ensure((size_t)na * 4));
        CK(W.dg_dcount.ensure(16 * 8));
        DigiScratch& D = W.dg;
        D.idx_a = W.dg_idx_a.as<uint32_t>(); D.idx_b = W.dg_idx_b.as<uint32_t>();
        D.key_a = W.dg_key_a.as<uint64_t>(); D.key_b = W.dg_key_b.as<uint64_t>();
        D.torder = W.dg_torder.as<uint32_t>(); D.flags = W.dg_flags.as<uint32_t>(); D.site = W.dg_site.as<int32_t>();
        D.hist = W.dg_hist.as<uint32_t>(); D.scan_aux = W.dg_aux.as<uint32_t>(); D.sel = W.dg_sel.as<uint32_t>();
        float* B = W.dg_blur.as<float>();
        D.Eb = B; D.xb = B + cap; D.yb = B + 2 * cap; D.zb = B + 3 * cap;
        D.single_idx = W.dg_single.as<uint32_t>();
        D.wcount = W.dg_wcount.as<uint32_t>(); D.wend = W.dg_wend.as<uint32_t>();
        D.dcount = W.dg_dcount.as<unsigned long long>();
        D.cap = cap;
        D.hist_cap = 256 * nb;
    }
    return GPET_OK;
}

static DigiParams digi_params(const gpet_ctx* c)
{
    DigiParams p{};
    p.key0 = (uint32_t)c->seed;
    p.key1 = (uint32_t)(c->seed >> 32) + c->sim_id;
    const Config& f = c->cfg;
    p.blurpolicy = f.blurpolicy; p.Eref = f.eref; p.Rref = f.rref; p.Eslope = f.eslope; p.Sblur = f.sblur;
    p.Eth = f.eth; p.dlevel = f.dlevel; p.dtype = f.dtype; p.tau = (double)f.dtime;
    p.ewin_lo = f.ewin_lo; p.ewin_hi = f.ewin_hi;
    p.window = c->coinc_window_ns * 1e-3;
    p.coinc_policy = c->coinc_policy;
    p.moduleN = c->geo.moduleN; p.crystalN = c->geo.crystalN;
    return p;
}

static void fill_stats(const Counters& h, gpet_run_stats* st)
{
    st->n_pairs = (int64_t)h.pairs;
    st->n_entered = (int64_t)h.entered;
    st->n_pulses = (int64_t)h.n_pulse;
    st->n_hits = (int64_t)h.n_hit;
    st->n_threshold = (int64_t)h.n_thr;
    st->n_deadtime = (int64_t)h.n_dead;
    st->n_singles = (int64_t)h.n_single;
    st->n_true = (int64_t)h.n_true;
    st->n_scatter = (int64_t)h.n_scat;
    st->n_random = (int64_t)h.n_rand;
    st->n_coinc = (int64_t)(h.n_true + h.n_scat + h.n_rand);
    st->n_multiple = (int64_t)h.n_mult;
    st->n_overflow = (int64_t)h.overflow;
    st->n_stepcap = (int64_t)h.stepcap;
    st->phantom_steps = (int64_t)h.ph_steps;
    st->detector_steps = (int64_t)h.det_steps;
    st->n_surrogate = (int64_t)h.n_surrogate;
    st->n_noise = (int64_t)h.n_noise;
}

// the leader's Work for a new run: reused unless other contexts still hold
// results in it
// stream s waits for the asynchronous copies of c, which read c's results:
// launches that rewrite those buffers go after them
static cudaError_t join_copies(gpet_ctx* c, cudaStream_t s)
{
    for (Staged* g : {&c->st_singles, &c->st_coinc})
        if (g->pending) {
            cudaError_t e = cudaStreamWaitEvent(s, g->done, 0);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

static Work& fresh_work(gpet_ctx* c)
{
    if (!c->work || c->work.use_count() > 1) c->work = std::make_shared<Work>();
    return *c->work;
}

// background singles of every simulation whose context asks for them,
// appended after W's first W.n_pulses pulses; sets W.n_digi
static int add_noise(gpet_ctx* c, Work& W, gpet_ctx* const* cs, int nsim, int64_t* launches)
{
    int64_t nd = W.n_pulses;
    for (int s = 0; s < nsim; ++s) {
        const gpet_ctx* x = cs[s];
        if (!(x->noise_lambda_us > 0.0f)) continue;
        NoiseParams np{};
        np.key0 = (uint32_t)x->seed;
        np.key1 = (uint32_t)(x->seed >> 32) + x->sim_id;
        np.lambda_us = x->noise_lambda_us;
        np.emean = x->noise_emean;
        np.sigma = x->noise_sigma;
        np.t0_us = (double)x->tstart * 1e6;
        np.t1_us = (double)x->tend * 1e6;
        np.interval_us = x->noise_interval_us;
        np.nint = np.t1_us > np.t0_us ? (int64_t)std::ceil((np.t1_us - np.t0_us) / np.interval_us) : 0;
        np.npanels = x->geo.npanels;
        np.moduleN = x->geo.moduleN;
        np.crystalN = x->geo.crystalN;
        np.sim = s;
        if (np.nint <= 0) continue;
        int rc = ensure_digi(c, W, std::max<int64_t>(np.nint, nd));
        if (rc) return rc;
        int64_t tot = 0;
        if (noise_count(np, W.dg, c->stream, launches, &tot)) return fail(c, GPET_ERR_CUDA, "background singles (count)");
        rc = grow_pulses(c, W, nd + tot, nd);
        if (rc) return rc;
        PulseDev P = pulse_view(W);
        if (noise_write(np, W.dg, P, nd, W.cnt.as<Counters>(), c->stream, launches))
            return fail(c, GPET_ERR_CUDA, "background singles (write)");
        nd += tot;
    }
    W.n_digi = nd;
    return GPET_OK;
}

// digitize W's pulses for nsims simulations with parameters prms (host),
// leaving per-simulation counts in W.hcnt and result offsets in W.s_off/c_off
static int digitize_work(gpet_ctx* c, Work& W, const std::vector<DigiParams>& prms,
                         gpet_run_stats* st, float* ms_digi)
{
    const int n = (int)prms.size();
    int rc = ensure_digi(c, W, W.n_digi);
    if (rc) return rc;
    CK(W.prms.ensure(sizeof(DigiParams) * n));
    CK(cudaMemcpyAsync(W.prms.p, prms.data(), sizeof(DigiParams) * n, cudaMemcpyHostToDevice, c->stream));
    PulseDev P = pulse_view(W);
    cudaEventRecord(c->ev[4], c->stream);
    int64_t ns = 0, nc = 0;
    rc = digitize_device(P, W.n_digi, W.prms.as<DigiParams>(), n, W.dg, W.cnt.as<Counters>(), c->stream,
                         &st->kernel_launches, &ns, &nc);
    if (rc) return fail(c, rc, std::string("digitizer failed: ") + cudaGetErrorString(cudaGetLastError()));
    cudaEventRecord(c->ev[5], c->stream);
    CK(cudaEventSynchronize(c->ev[5]));
    cudaEventElapsedTime(ms_digi, c->ev[4], c->ev[5]);
    W.hcnt.assign(n, Counters{});
    CK(cudaMemcpy(W.hcnt.data(), W.cnt.p, sizeof(Counters) * n, cudaMemcpyDeviceToHost));
    W.n_singles = ns;
    W.n_coinc = nc;
    W.s_off.assign(n + 1, 0);
    W.c_off.assign(n + 1, 0);
    for (int s = 0; s < n; ++s) {
        W.s_off[s + 1] = W.s_off[s] + (int64_t)W.hcnt[s].n_single;
        W.c_off[s + 1] = W.c_off[s] + (int64_t)(W.hcnt[s].n_true + W.hcnt[s].n_scat + W.hcnt[s].n_rand);
    }
    if (W.s_off[n] != ns || W.c_off[n] != nc) return fail(c, GPET_ERR_CUDA, "digitizer counts are inconsistent");
    return GPET_OK;
}

// Everything the launches of one chunk depend on. Two chunks with equal
// ChunkLaunch values issue identical launches (the waves themselves are read
// from the device table at run time), so one instantiated CUDA graph serves
// both; the struct is zero-filled before use so it compares bytewise.
struct ChunkLaunch {
    const Wave* d_waves;
    unsigned long long* d_work;
    unsigned long long* qcount;
    PairBuf pb;
    QueueDev q;
    Counters* dcnt;
    const cudaEvent_t* ev;        // 3 per wave
    size_t smem;
    int32_t nwaves;
    int32_t multi;
    uint32_t src_blocks, src_threads, ph_blocks, walk_blocks;
    int32_t period;
    int32_t graph;
};

static cudaError_t enqueue_chunk(const ChunkLaunch& L, cudaStream_t s)
{
    const unsigned flag = L.graph ? cudaEventRecordExternal : cudaEventRecordDefault;
    cudaError_t e;
    if ((e = cudaMemsetAsync(L.qcount, 0, 8, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(L.d_work, 0, 64 * (size_t)L.nwaves, s)) != cudaSuccess) return e;
    for (int k = 0; k < L.nwaves; ++k) {
        if ((e = cudaEventRecordWithFlags(L.ev[3 * k], s, flag)) != cudaSuccess) return e;
        if ((e = launch_source(L.multi != 0, L.src_blocks, L.src_threads, L.smem, s, L.d_waves, k, L.pb, L.dcnt)) !=
            cudaSuccess)
            return e;
        if ((e = launch_walk(L.multi != 0, L.walk_blocks, s, L.d_waves, k, L.pb)) != cudaSuccess) return e;
        if ((e = cudaEventRecordWithFlags(L.ev[3 * k + 1], s, flag)) != cudaSuccess) return e;
        if ((e = launch_phantom(L.multi != 0, L.ph_blocks, L.smem, s, L.d_waves, k, L.pb, L.q, L.dcnt, L.period)) !=
            cudaSuccess)
            return e;
        if ((e = cudaEventRecordWithFlags(L.ev[3 * k + 2], s, flag)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// the chunk's launches: replayed from the cached graph when nothing they
// depend on changed, captured and instantiated again otherwise
static int launch_chunk(gpet_ctx* c, Work& W, const ChunkLaunch& L, int slot)
{
    if (!L.graph) {
        CK(enqueue_chunk(L, c->stream));
        return GPET_OK;
    }
    const unsigned char* key = reinterpret_cast<const unsigned char*>(&L);
    cudaGraphExec_t& gexec = W.gexec[slot];
    std::vector<unsigned char>& gkey = W.gkey[slot];
    if (!gexec || gkey.size() != sizeof(L) || std::memcmp(gkey.data(), key, sizeof(L)) != 0) {
        if (gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        gkey.clear();
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = enqueue_chunk(L, c->stream);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gexec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            gexec = nullptr;
            return cuda_fail(c, e, "capture of the chunk's launches");
        }
        gkey.assign(key, key + sizeof(L));
    }
    CK(cudaGraphLaunch(gexec, c->stream));
    return GPET_OK;
}

// one wave: decays [g, g + n) of the batch's concatenated decay list
struct WaveH {
    int64_t g, n;
    int first_seg, nseg;
};

// limit >= 0 runs only the first `limit` decays of each simulation;
// transport_only stops after the detector stage (no digitizer, no results),
// stats[0] receiving the stage times: the autotuner's measurement
static int run_batch(gpet_ctx* const* cs, int nsim, gpet_run_stats* stats, int64_t limit = -1,
                     bool transport_only = false)
{
    gpet_ctx* c = cs[0];
    for (int s = 0; s < nsim; ++s) {
        gpet_ctx* x = cs[s];
        if (!x) return fail(c, GPET_ERR_ARG, "null context in the batch");
        if (!x->have_tables || !x->have_phantom || !x->have_geo || !x->have_source)
            return fail(x, GPET_ERR_ARG, "tables, phantom, geometry and source must be set before a run");
        if (x->device != c->device) return fail(c, GPET_ERR_ARG, "a batch must be on one device");
        for (int r = 0; r < s; ++r)
            if (cs[r] == x) return fail(c, GPET_ERR_ARG, "a context appears twice in the batch");
    }
    if (nsim > 1)
        for (int s = 0; s < nsim; ++s) {
            if (cs[s]->record_exits) return fail(c, GPET_ERR_ARG, "record_exits is for single runs");
            if (cs[s]->record_entries) return fail(c, GPET_ERR_ARG, "record_entries is for single runs");
            if (cs[s]->record_source) return fail(c, GPET_ERR_ARG, "record_source is for single runs");
            if (cs[s]->sur != c->sur) return fail(c, GPET_ERR_ARG, "the simulations of a batch share one surrogate or none");
        }
    CK(cudaSetDevice(c->device));
    // a run that fails leaves no results (the record arrays are then partly written)
    for (int s = 0; s < nsim; ++s) cs[s]->have_results = false;
    // nothing of an earlier run may still use the work buffers
    CK(cudaStreamSynchronize(c->stream2));
    std::vector<int64_t> nd(nsim);
    int64_t ND = 0;
    bool rec_hits = false;
    size_t smem = 0;
    for (int s = 0; s < nsim; ++s) {
        int rc = build_sim(cs[s]);
        if (rc) return rc;
        nd[s] = total_decays(cs[s]);
        if (limit >= 0) nd[s] = std::min(nd[s], limit);
        ND += nd[s];
        rec_hits = rec_hits || cs[s]->record_hits;
        smem = std::max(smem, (size_t)cs[s]->geo.npanels * kPanelStride * 4);
    }
    Work& W = fresh_work(c);
    // the detector stage rewrites the pulses that copies of the last results
    // may still be reading (the transport before it overlaps those copies)
    CK(join_copies(c, c->stream2));
    W.nsims = nsim;
    W.n_pulses = W.n_hits = W.n_singles = W.n_coinc = 0;
    W.sim_hits.assign(nsim, 0);
    for (int s = 0; s < nsim; ++s) W.sim_hits[s] = cs[s]->record_hits ? 1 : 0;
    // descriptors of the batch
    std::vector<SimDesc> sims(nsim);
    std::vector<DigiParams> prms(nsim);
    for (int s = 0; s < nsim; ++s) { sims[s] = cs[s]->sim; prms[s] = digi_params(cs[s]); }
    CK(W.sims.ensure(sizeof(SimDesc) * nsim));
    CK(cudaMemcpyAsync(W.sims.p, sims.data(), sizeof(SimDesc) * nsim, cudaMemcpyHostToDevice, c->stream));
    CK(W.cnt.ensure(sizeof(Counters) * nsim));
    CK(cudaMemsetAsync(W.cnt.p, 0, sizeof(Counters) * nsim, c->stream));
    CK(W.aux.ensure(64 * 8));
    CK(cudaMemsetAsync(W.aux.p, 0, 64 * 8, c->stream));
    // waves of at most `sub` decays (and kMaxSeg simulations), chunks of at most `chunk` decays
    const int64_t sub = std::min(c->sub_decays, std::max<int64_t>(ND, 1));
    const int64_t chunk = std::max(std::min(c->chunk_decays, std::max<int64_t>(ND, 1)), sub);
    std::vector<int64_t> seg_g0, seg_d0;
    std::vector<int32_t> seg_sim;
    std::vector<WaveH> waves;
    {
        int s = 0;
        int64_t ds = 0;   // next decay of simulation s
        int64_t g = 0;
        while (s < nsim && ds >= nd[s]) { s++; ds = 0; }
        while (s < nsim) {
            WaveH wv{g, 0, (int)seg_sim.size(), 0};
            while (s < nsim && wv.n < sub && wv.nseg < kMaxSeg) {
                int64_t take = std::min(nd[s] - ds, sub - wv.n);
                seg_g0.push_back(wv.n);
                seg_d0.push_back(ds);
                seg_sim.push_back(s);
                wv.nseg++;
                wv.n += take;
                ds += take;
                if (ds >= nd[s]) { s++; ds = 0; while (s < nsim && ds >= nd[s]) s++; }
            }
            g += wv.n;
            waves.push_back(wv);
        }
    }
    // per wave: g0[nseg + 1], d0[nseg], sim[nseg], laid out one wave after another
    std::vector<int64_t> wg0, wd0;
    std::vector<int32_t> wsim;
    std::vector<size_t> woff_g0(waves.size()), woff_d0(waves.size());
    for (size_t w = 0; w < waves.size(); ++w) {
        woff_g0[w] = wg0.size();
        woff_d0[w] = wd0.size();
        for (int k = 0; k < waves[w].nseg; ++k) {
            wg0.push_back(seg_g0[waves[w].first_seg + k]);
            wd0.push_back(seg_d0[waves[w].first_seg + k]);
            wsim.push_back(seg_sim[waves[w].first_seg + k]);
        }
        wg0.push_back(waves[w].n);
    }
    const size_t seg_bytes = (wg0.size() + wd0.size()) * 8 + wsim.size() * 4 + 64;
    CK(W.segs.ensure(seg_bytes));
    int64_t* d_g0 = W.segs.as<int64_t>();
    int64_t* d_d0 = d_g0 + wg0.size();
    int32_t* d_sim = reinterpret_cast<int32_t*>(d_d0 + wd0.size());
    if (!wg0.empty()) CK(cudaMemcpyAsync(d_g0, wg0.data(), wg0.size() * 8, cudaMemcpyHostToDevice, c->stream));
    if (!wd0.empty()) CK(cudaMemcpyAsync(d_d0, wd0.data(), wd0.size() * 8, cudaMemcpyHostToDevice, c->stream));
    if (!wsim.empty()) CK(cudaMemcpyAsync(d_sim, wsim.data(), wsim.size() * 4, cudaMemcpyHostToDevice, c->stream));
    // buffers
    if (2 * chunk > W.q_cap) {
        CK(W.q_f.ensure((size_t)2 * chunk * 7 * 4));
        CK(W.q_t.ensure((size_t)2 * chunk * 8));
        CK(W.q_i.ensure((size_t)2 * chunk * 5 * 4));
        CK(W.qb_f.ensure((size_t)2 * chunk * 7 * 4));
        CK(W.qb_t.ensure((size_t)2 * chunk * 8));
        CK(W.qb_i.ensure((size_t)2 * chunk * 5 * 4));
        W.q_cap = 2 * chunk;
    }
    if (c->sur) {
        CK(W.q2_f.ensure((size_t)W.q_cap * 7 * 4));
        CK(W.q2_t.ensure((size_t)W.q_cap * 8));
        CK(W.q2_i.ensure((size_t)W.q_cap * 5 * 4));
        CK(W.sidx.ensure((size_t)W.q_cap * 4));
    }
    if (c->record_entries && !transport_only) CK(W.ent.ensure((size_t)W.q_cap * sizeof(EntryRec)));
    if (sub > W.pb_cap) {
        CK(W.pb_f.ensure((size_t)sub * 11 * 4));
        CK(W.pb_t.ensure((size_t)sub * 8));
        CK(W.pb_n.ensure((size_t)sub));
        CK(W.pb_wf.ensure((size_t)sub * kWalkLists * kWalkFields * 4));
        CK(W.pb_wj.ensure((size_t)sub * kWalkLists * 4));
        W.pb_cap = sub;
    }
    int rc = grow_pulses(c, W, 1 << 20, 0);
    if (rc) return rc;
    if (rec_hits) { rc = grow_hits(c, W, 1 << 20, 0); if (rc) return rc; }
    const bool rec_exits = c->record_exits && !transport_only;
    const bool rec_entries = c->record_entries && !transport_only;
    c->host_entries.clear();
    const bool rec_source = c->record_source && !transport_only;
    if (rec_source) {
        CK(W.source.ensure((size_t)2 * chunk * sizeof(SrcRec)));
        CK(c->host_source.resize((size_t)2 * ND));   // every slot is copied from the device
    } else {
        c->host_source.clear();
    }
    // the learned detector response, checked against every simulation's detector
    SurrogateDev sdev{};
    const bool use_sur = c->sur != nullptr;
    if (use_sur) {
        for (int s = 0; s < nsim; ++s) {
            SurGeom g{};
            int r2 = ctx_geometry(cs[s], &g);
            if (r2) return fail(c, r2, "no detector geometry");
            const char* why = "";
            if (surrogate_view(c->sur, g, &sdev, &why)) return fail(cs[s], GPET_ERR_ARG, why);
        }
        CK(W.serr.ensure(4));
        CK(cudaMemsetAsync(W.serr.p, 0, 4, c->stream));
    }
    if (rec_exits) {
        CK(W.exits.ensure((size_t)2 * chunk * sizeof(ExitRec)));
        CK(c->host_exits.resize((size_t)2 * ND));   // every slot is copied from the device
    } else {
        c->host_exits.clear();
    }
    PairBuf pb;
    pb.f = W.pb_f.as<float>(); pb.t = W.pb_t.as<double>(); pb.nph = W.pb_n.as<uint8_t>(); pb.cap = W.pb_cap;
    pb.wf = W.pb_wf.as<float>(); pb.wj = W.pb_wj.as<int32_t>();
    Counters* dcnt = W.cnt.as<Counters>();
    unsigned long long* pcount = W.aux.as<unsigned long long>() + 1;
    unsigned long long* hcount = W.aux.as<unsigned long long>() + 2;
    const bool multi = nsim > 1;
    // one simulation: its panels are staged in shared memory
    if (multi) smem = 0;
    else CK(transport_set_smem(smem));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    int bps = 0;
    CK(phantom_blocks_per_sm(multi, smem, &bps));
    int det_bps = 0;
    CK(detector_blocks_per_sm(multi, (unsigned)c->det_threads, smem, &det_bps));
    det_bps = std::max(det_bps, 1);
    unsigned long long* dtake = W.aux.as<unsigned long long>() + 8;
    bps = std::max(1, bps);
    if (c->phantom_bps > 0) bps = std::min(bps, c->phantom_bps);
    int walk_bps = 0;
    CK(walk_blocks_per_sm(multi, &walk_bps));
    walk_bps = std::max(walk_bps, 1);
    const SimDesc* d_sims = W.sims.as<SimDesc>();
    // wave table and counters for the largest chunk
    size_t max_k = 1;
    for (size_t w0 = 0; w0 < waves.size();) {
        size_t w1 = w0;
        while (w1 < waves.size() && waves[w1].g + waves[w1].n - waves[w0].g <= chunk) w1++;
        if (w1 == w0) w1 = w0 + 1;
        max_k = std::max(max_k, w1 - w0);
        w0 = w1;
    }
    CK(W.d_waves.ensure(max_k * sizeof(Wave)));
    CK(W.d_work.ensure(max_k * 64));
    if (W.h_waves_cap < max_k) {
        if (W.h_waves) cudaFreeHost(W.h_waves);
        W.h_waves = nullptr;
        W.h_waves_cap = 0;
        CK(cudaMallocHost(reinterpret_cast<void**>(&W.h_waves), max_k * sizeof(Wave)));
        W.h_waves_cap = max_k;
    }
    while (W.tev.size() < 3 * max_k) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        W.tev.push_back(e);
    }
    gpet_run_stats tot{};
    float ms_det = 0, ms_src = 0, ms_ph = 0, ms_sur = 0;
    cudaEventRecord(c->ev[0], c->stream);
    // Chunks alternate between two queues. Chunk k's detector stage runs on
    // stream2 while chunk k+1's source and phantom waves run on the main
    // stream; chunk k+2's transport waits until that detector stage is done
    // with the queue. Pulse and hit buffers are checked against an upper
    // bound (their count so far plus the worst case of the chunks in flight),
    // and grown only with stream2 idle.
    int64_t pulses_used = 0, hits_used = 0;
    int64_t inflight = 0;        // queue length of the detector stage that may still run
    size_t wi = 0;
    int ci = 0;
    while (wi < waves.size()) {
        const int b = ci & 1;
        // one chunk: waves until `chunk` decays
        const int64_t cg0 = waves[wi].g;
        size_t we = wi;
        while (we < waves.size() && waves[we].g + waves[we].n - cg0 <= chunk) we++;
        if (we == wi) we = wi + 1;
        const int K = (int)(we - wi);
        for (int k = 0; k < K; ++k) {
            const size_t w = wi + k;
            Wave& wave = W.h_waves[k];
            wave.sims = d_sims;
            wave.g0 = d_g0 + woff_g0[w];
            wave.d0 = d_d0 + woff_d0[w];
            wave.sim = d_sim + woff_d0[w];
            wave.nseg = waves[w].nseg;
            wave.n = waves[w].n;
            wave.work = W.d_work.as<unsigned long long>() + 8 * k;          // 8 counters per wave:
            wave.walkn = W.d_work.as<unsigned long long>() + 8 * k + 1;     // photons, walk lists
            wave.exits = rec_exits ? W.exits.as<ExitRec>() + 2 * (waves[w].g - cg0) : nullptr;
            wave.source = rec_source ? W.source.as<SrcRec>() + 2 * (waves[w].g - cg0) : nullptr;
        }
        CK(cudaMemcpyAsync(W.d_waves.p, W.h_waves, K * sizeof(Wave), cudaMemcpyHostToDevice, c->stream));
        unsigned long long* qcount = W.aux.as<unsigned long long>() + (b ? 6 : 0);
        QueueDev q;
        q.f = (b ? W.qb_f : W.q_f).as<float>(); q.t = (b ? W.qb_t : W.q_t).as<double>();
        q.i = (b ? W.qb_i : W.q_i).as<int32_t>();
        q.count = qcount; q.cap = W.q_cap;
        if (ci >= 2) CK(cudaStreamWaitEvent(c->stream, c->qev[2 + b], 0));   // the queue is free again
        ChunkLaunch L;
        std::memset(&L, 0, sizeof(L));
        L.d_waves = W.d_waves.as<Wave>();
        L.d_work = W.d_work.as<unsigned long long>();
        L.qcount = qcount;
        L.pb = pb;
        L.q = q;
        L.dcnt = dcnt;
        L.ev = W.tev.data();
        L.smem = smem;
        L.nwaves = K;
        L.multi = multi ? 1 : 0;
        L.src_threads = (uint32_t)c->src_threads;
        L.src_blocks = (uint32_t)std::max<int64_t>(1, std::min<int64_t>((sub + c->src_threads - 1) / c->src_threads,
                                                                      (int64_t)nsm * 32));
        L.ph_blocks = (uint32_t)(bps * nsm);
        L.walk_blocks = (uint32_t)(walk_bps * nsm);
        L.period = c->drain_period;
        L.graph = c->use_graphs ? 1 : 0;
        rc = launch_chunk(c, W, L, b);
        if (rc) return rc;
        tot.kernel_launches += 3 * K;
        CK(cudaEventRecord(c->qev[b], c->stream));
        unsigned long long hq3[3] = {0, 0, 0};   // queue, pulses and hits so far (lower bounds)
        CK(cudaMemcpyAsync(&hq3[0], qcount, 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(&hq3[1], pcount, 16, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaGetLastError());
        const unsigned long long hq = hq3[0];
        for (int e = 0; e < 3 * K; e += 3) {
            float a = 0, bb = 0;
            cudaEventElapsedTime(&a, W.tev[e], W.tev[e + 1]);
            cudaEventElapsedTime(&bb, W.tev[e + 1], W.tev[e + 2]);
            ms_src += a;
            ms_ph += bb;
        }
        const int64_t cn = waves[we - 1].g + waves[we - 1].n - cg0;
        if (rec_exits)
            CK(cudaMemcpyAsync(c->host_exits.data() + 2 * cg0, W.exits.p, (size_t)2 * cn * sizeof(ExitRec),
                               cudaMemcpyDeviceToHost, c->stream));
        if (rec_source)
            CK(cudaMemcpyAsync(c->host_source.data() + 2 * cg0, W.source.p, (size_t)2 * cn * sizeof(SrcRec),
                               cudaMemcpyDeviceToHost, c->stream));
        // room for the worst case of this chunk and of the one still in flight
        pulses_used = std::max<int64_t>(pulses_used, std::min<int64_t>((int64_t)hq3[1], W.p_cap));
        hits_used = std::max<int64_t>(hits_used, std::min<int64_t>((int64_t)hq3[2], W.h_cap));
        const int64_t need_p = pulses_used + (inflight + (int64_t)hq) * kMaxPulse;
        const int64_t need_h = hits_used + (inflight + (int64_t)hq) * kMaxHits;
        if (need_p > W.p_cap || (rec_hits && need_h > W.h_cap)) {
            CK(cudaStreamSynchronize(c->stream2));
            unsigned long long hp[2] = {0, 0};
            CK(cudaMemcpy(hp, pcount, 16, cudaMemcpyDeviceToHost));
            pulses_used = (int64_t)std::min<unsigned long long>(hp[0], (unsigned long long)W.p_cap);
            hits_used = (int64_t)std::min<unsigned long long>(hp[1], (unsigned long long)W.h_cap);
            inflight = 0;
            // leave room for two more chunks like this one
            rc = grow_pulses(c, W, pulses_used + 3 * (int64_t)hq * kMaxPulse, pulses_used);
            if (rc) return rc;
            if (rec_hits) {
                rc = grow_hits(c, W, hits_used + 3 * (int64_t)hq * kMaxHits, hits_used);
                if (rc) return rc;
            }
        }
        PulseDev P = pulse_view(W);
        P.sim = multi ? W.p_sim.as<int32_t>() : nullptr;
        HitDev H;
        H.id = W.h_id.as<int32_t>(); H.f = W.h_f.as<float>(); H.count = hcount; H.cap = W.h_cap;
        H.sim = multi ? W.h_sim.as<int32_t>() : nullptr;
        const int dt = c->det_threads;
        // persistent: at most the resident blocks, whose lanes take photons as they finish
        int64_t dblocks = std::min<int64_t>(((int64_t)hq + dt - 1) / dt, (int64_t)nsm * det_bps);
        EntryRec* ent = rec_entries ? W.ent.as<EntryRec>() : nullptr;
        while (W.dev.size() < 4 * (size_t)(ci + 1)) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            W.dev.push_back(e);
        }
        cudaStream_t s2 = c->stream2;
        CK(cudaStreamWaitEvent(s2, c->qev[b], 0));
        CK(cudaMemsetAsync(dtake, 0, 8, s2));
        q.take = dtake;
        cudaEventRecord(W.dev[4 * ci], s2);
        if (hq > 0 && use_sur) {
            // photons in the surrogate's domain take the learned response, the
            // others the Monte Carlo; the kernels read their counts on the device
            QueueDev q2;
            q2.f = W.q2_f.as<float>(); q2.t = W.q2_t.as<double>(); q2.i = W.q2_i.as<int32_t>();
            q2.count = W.aux.as<unsigned long long>() + 4; q2.cap = W.q_cap;
            unsigned long long* scount = W.aux.as<unsigned long long>() + 5;
            CK(cudaMemsetAsync(q2.count, 0, 16, s2));
            q2.take = dtake;
            CK(launch_route(sdev, q, (int64_t)hq, q2, W.sidx.as<uint32_t>(), scount, s2));
            CK(launch_detector(multi, (unsigned)std::max<int64_t>(dblocks, 1), (unsigned)dt, smem, s2, d_sims, q2, P,
                               H, rec_hits ? 1 : 0, dcnt, ent));
            cudaEventRecord(W.dev[4 * ci + 2], s2);
            CK(launch_surrogate(sdev, d_sims, q, W.sidx.as<uint32_t>(), scount, (int64_t)hq, P, dcnt,
                                W.serr.as<int>(), s2));
            cudaEventRecord(W.dev[4 * ci + 3], s2);
            tot.kernel_launches += 3;
        } else if (hq > 0) {
            CK(launch_detector(multi, (unsigned)std::max<int64_t>(dblocks, 1), (unsigned)dt, smem, s2, d_sims, q, P,
                               H, rec_hits ? 1 : 0, dcnt, ent));
            tot.kernel_launches++;
        }
        cudaEventRecord(W.dev[4 * ci + 1], s2);
        CK(cudaEventRecord(c->qev[2 + b], s2));
        if (rec_entries && hq > 0) {
            CK(cudaStreamSynchronize(s2));
            unsigned long long ne = hq;
            if (use_sur) CK(cudaMemcpy(&ne, W.aux.as<unsigned long long>() + 4, 8, cudaMemcpyDeviceToHost));
            const size_t old = c->host_entries.size();
            c->host_entries.resize(old + (size_t)ne);
            CK(cudaMemcpy(c->host_entries.data() + old, W.ent.p, (size_t)ne * sizeof(EntryRec),
                          cudaMemcpyDeviceToHost));
        }
        inflight = (int64_t)hq;
        wi = we;
        ci++;
    }
    // join the detector stream
    CK(cudaStreamSynchronize(c->stream2));
    CK(cudaGetLastError());
    CK(join_copies(c, c->stream));
    {
        unsigned long long hp[2] = {0, 0};
        CK(cudaMemcpy(hp, pcount, 16, cudaMemcpyDeviceToHost));
        pulses_used = (int64_t)std::min<unsigned long long>(hp[0], (unsigned long long)W.p_cap);
        hits_used = (int64_t)std::min<unsigned long long>(hp[1], (unsigned long long)W.h_cap);
    }
    for (int k = 0; k < ci; ++k) {
        float ms = 0;
        cudaEventElapsedTime(&ms, W.dev[4 * k], W.dev[4 * k + 1]);
        ms_det += ms;
        if (use_sur) {
            cudaEventElapsedTime(&ms, W.dev[4 * k + 2], W.dev[4 * k + 3]);
            ms_sur += ms;
        }
    }
    Counters h0{};
    CK(cudaMemcpy(&h0, dcnt, sizeof(Counters), cudaMemcpyDeviceToHost));
    if (h0.queue_drop || h0.pulse_drop || h0.hit_drop)
        return fail(c, GPET_ERR_CAPACITY, "a device buffer overflowed (queue/pulse/hit drops)");
    if (use_sur) {
        int herr = 0;
        CK(cudaMemcpy(&herr, W.serr.p, 4, cudaMemcpyDeviceToHost));
        if (herr) return fail(c, GPET_ERR_CUDA, "a tensor-core wait of the surrogate gave up");
    }
    W.n_pulses = pulses_used;
    W.n_hits = rec_hits ? hits_used : 0;
    if (transport_only) {
        // results of this partial run are not kept
        for (int s = 0; s < nsim; ++s) cs[s]->have_results = false;
        cudaEventRecord(c->ev[3], c->stream);
        CK(cudaEventSynchronize(c->ev[3]));
        float ms_wall = 0;
        cudaEventElapsedTime(&ms_wall, c->ev[0], c->ev[3]);
        if (stats) {
            stats[0] = tot;
            stats[0].ms_total = ms_wall;
            stats[0].ms_source = ms_src;
            stats[0].ms_phantom = ms_ph;
            stats[0].ms_source_phantom = ms_src + ms_ph;
            stats[0].ms_detector = ms_det;
            stats[0].n_pulses = pulses_used;
        }
        return GPET_OK;
    }
    rc = add_noise(c, W, cs, nsim, &tot.kernel_launches);
    if (rc) return rc;
    float ms_digi = 0;
    rc = digitize_work(c, W, prms, &tot, &ms_digi);
    if (rc) return rc;
    cudaEventRecord(c->ev[3], c->stream);
    CK(cudaEventSynchronize(c->ev[3]));
    float ms_tot = 0;
    cudaEventElapsedTime(&ms_tot, c->ev[0], c->ev[3]);
    for (int s = 0; s < nsim; ++s) {
        gpet_run_stats st = tot;
        fill_stats(W.hcnt[s], &st);
        if (!W.sim_hits[s]) st.n_hits = 0;
        st.n_decays = nd[s];
        st.ms_total = ms_tot;
        st.ms_source_phantom = ms_src + ms_ph;
        st.ms_source = ms_src;
        st.ms_phantom = ms_ph;
        st.ms_detector = ms_det;
        st.ms_surrogate = ms_sur;
        st.ms_digitizer = ms_digi;
        st.ms_coincidence = 0;
        cs[s]->work = c->work;
        cs[s]->res_sim = s;
        cs[s]->have_results = true;
        cs[s]->last = st;
        if (s > 0) cs[s]->host_exits.clear();
        if (stats) stats[s] = st;
    }
    return GPET_OK;
}

// ---------------------------------------------------------------- autotuner
// Launch-shape parameters of the transport: none of them changes a result
// (every random stream is keyed by decay, photon and pulse, and every output
// is put in a total order), only the time.
struct Shape {
    int64_t sub, chunk;
    int bps, period, det_threads, src_threads;
};

static Shape get_shape(const gpet_ctx* c)
{
    return {c->sub_decays, c->chunk_decays, c->phantom_bps, c->drain_period, c->det_threads, c->src_threads};
}

static void set_shape(gpet_ctx* c, const Shape& s)
{
    c->sub_decays = s.sub; c->chunk_decays = s.chunk; c->phantom_bps = s.bps; c->drain_period = s.period;
    c->det_threads = s.det_threads; c->src_threads = s.src_threads;
}

// transport time (source + phantom + detector, device) of the first `sample`
// decays with the context's current shape: the best of `reps` runs
static int time_transport(gpet_ctx* c, int64_t sample, int reps, double* ms)
{
    gpet_ctx* one[1] = {c};
    double best = 1e30;
    for (int r = 0; r < reps; ++r) {
        gpet_run_stats st{};
        int rc = run_batch(one, 1, &st, sample, true);
        if (rc) return rc;
        best = std::min(best, st.ms_total);
    }
    *ms = best;
    return GPET_OK;
}

// Coordinate descent over the shape, one parameter at a time, each candidate
// timed on the same sample of the context's own workload.
static int autotune(gpet_ctx* c, int64_t sample, gpet_tuning* out)
{
    if (!c->have_tables || !c->have_phantom || !c->have_geo || !c->have_source)
        return fail(c, GPET_ERR_ARG, "tables, phantom, geometry and source must be set before tuning");
    gpet_ctx* one[1] = {c};
    (void)one;
    int rc = build_sim(c);
    if (rc) return rc;
    const int64_t total = total_decays(c);
    if (sample <= 0) sample = std::min<int64_t>(total, 1ll << 24);
    sample = std::min(sample, total);
    const Shape start = get_shape(c);
    if (sample < 4096) {
        if (out) std::memset(out, 0, sizeof(*out));
        c->tuned = true;
        return GPET_OK;
    }
    int cands = 0;
    double best_ms = 0;
    rc = time_transport(c, sample, 1, &best_ms);   // warm-up: buffers, graph, caches
    if (rc) { set_shape(c, start); return rc; }
    rc = time_transport(c, sample, 2, &best_ms);
    if (rc) { set_shape(c, start); return rc; }
    const double ms_default = best_ms;
    Shape best = start;
    cands++;
    auto consider = [&](Shape cand) -> int {
        set_shape(c, cand);
        double ms = 0;
        int r = time_transport(c, sample, 2, &ms);
        cands++;
        if (r) return r;
        if (ms < best_ms * 0.995) {
            best_ms = ms;
            best = cand;
        }
        set_shape(c, best);
        return GPET_OK;
    };
    for (int64_t sub : {1ll << 19, 1ll << 20, 1ll << 21, 1ll << 22, 1ll << 23, 1ll << 24}) {
        if (sub == best.sub || sub > sample) continue;
        Shape t = best; t.sub = sub; t.chunk = std::max(t.chunk, sub);
        if ((rc = consider(t))) break;
    }
    int maxb = 0;
    if (!rc && phantom_blocks_per_sm(false, (size_t)c->geo.npanels * kPanelStride * 4, &maxb) == cudaSuccess)
        for (int b = maxb - 1; b >= std::max(1, maxb - 2) && !rc; --b) {
            Shape t = best; t.bps = b;
            rc = consider(t);
        }
    for (int p : {24, 16, 8}) {
        if (rc || p == best.period) continue;
        Shape t = best; t.period = p;
        rc = consider(t);
    }
    for (int th : {128, 64}) {
        if (rc || th == best.det_threads) continue;
        Shape t = best; t.det_threads = th;
        rc = consider(t);
    }
    for (int th : {128}) {
        if (rc || th == best.src_threads) continue;
        Shape t = best; t.src_threads = th;
        rc = consider(t);
    }
    for (int64_t ch : {sample / 4, sample / 2}) {
        if (rc || ch < best.sub || ch < 1024 || ch == best.chunk) continue;
        Shape t = best; t.chunk = ch;
        rc = consider(t);
    }
    if (rc) { set_shape(c, start); return rc; }
    set_shape(c, best);
    c->tuned = true;
    if (out) {
        out->sub_decays = best.sub;
        out->chunk_decays = best.chunk;
        out->phantom_blocks_per_sm = best.bps;
        out->drain_period = best.period;
        out->detector_threads = best.det_threads;
        out->source_threads = best.src_threads;
        out->candidates = cands;
        out->sample_decays = sample;
        out->ms_default = ms_default;
        out->ms_tuned = best_ms;
    }
    return GPET_OK;
}

extern "C" {

int gpet_run(gpet_ctx* c, gpet_run_stats* st)
{
    if (!c) return GPET_ERR_ARG;
    if (c->autotune && !c->tuned) {
        int rc = autotune(c, 0, nullptr);
        if (rc) return rc;
    }
    gpet_ctx* one[1] = {c};
    return run_batch(one, 1, st);
}

int gpet_autotune(gpet_ctx* c, int64_t sample_decays, gpet_tuning* out)
{
    if (!c) return GPET_ERR_ARG;
    CK(cudaSetDevice(c->device));
    return autotune(c, sample_decays, out);
}

int gpet_run_batched(gpet_ctx* const* ctxs, int32_t n, gpet_run_stats* stats)
{
    if (!ctxs || n < 1 || !ctxs[0]) return GPET_ERR_ARG;
    return run_batch(ctxs, n, stats);
}

int gpet_digitize(gpet_ctx* c, const gpet_event* ev, const uint8_t* scat, const uint8_t* slot, int64_t n,
                  gpet_run_stats* st)
{
    if (!c || n < 0 || (n > 0 && (!ev || !scat || !slot))) return GPET_ERR_ARG;
    if (!c->have_geo) return fail(c, GPET_ERR_ARG, "load the geometry first (site numbering)");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream2));
    gpet_run_stats local{};
    if (!st) st = &local;
    std::memset(st, 0, sizeof(*st));
    Work& W = fresh_work(c);
    CK(join_copies(c, c->stream));
    W.nsims = 1;
    W.sim_hits.assign(1, 0);
    int rc = grow_pulses(c, W, std::max<int64_t>(n, 1), 0);
    if (rc) return rc;
    CK(W.cnt.ensure(sizeof(Counters)));
    CK(cudaMemsetAsync(W.cnt.p, 0, sizeof(Counters), c->stream));
    CK(W.aux.ensure(64 * 8));
    std::vector<int32_t> I((size_t)n * 6);
    std::vector<double> T((size_t)n);
    std::vector<float> F((size_t)n * 4);
    std::vector<uint8_t> M((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        I[i] = ev[i].parn; I[n + i] = ev[i].pann; I[2 * n + i] = ev[i].modn; I[3 * n + i] = ev[i].cryn;
        I[4 * n + i] = ev[i].siten; I[5 * n + i] = ev[i].eventid;
        T[i] = ev[i].t;
        F[i] = ev[i].E; F[n + i] = ev[i].x; F[2 * n + i] = ev[i].y; F[3 * n + i] = ev[i].z;
        if (slot[i] > 0x7f) return fail(c, GPET_ERR_ARG, "slot must be < 128");
        M[i] = (uint8_t)(slot[i] | (scat[i] ? 0x80 : 0));
    }
    for (int a = 0; a < 6; ++a)
        CK(cudaMemcpyAsync(W.p_int.as<int32_t>() + a * W.p_cap, I.data() + a * n, n * 4, cudaMemcpyHostToDevice,
                           c->stream));
    CK(cudaMemcpyAsync(W.p_t.p, T.data(), n * 8, cudaMemcpyHostToDevice, c->stream));
    for (int a = 0; a < 4; ++a)
        CK(cudaMemcpyAsync(W.p_f.as<float>() + a * W.p_cap, F.data() + a * n, n * 4, cudaMemcpyHostToDevice,
                           c->stream));
    CK(cudaMemcpyAsync(W.p_meta.p, M.data(), n, cudaMemcpyHostToDevice, c->stream));
    W.n_pulses = n;
    W.n_hits = 0;
    gpet_ctx* one[1] = {c};
    rc = add_noise(c, W, one, 1, &st->kernel_launches);
    if (rc) return rc;
    std::vector<DigiParams> prms(1, digi_params(c));
    float ms_digi = 0;
    rc = digitize_work(c, W, prms, st, &ms_digi);
    if (rc) return rc;
    fill_stats(W.hcnt[0], st);
    st->n_pulses = n;
    st->ms_digitizer = ms_digi;
    st->ms_total = ms_digi;
    c->res_sim = 0;
    c->have_results = true;
    c->host_exits.clear();
    c->last = *st;
    return GPET_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- outputs
// Event records of pulses: `idx` lists pulse indices (device) or NULL for all
static int gather(gpet_ctx* c, Work& W, const uint32_t* d_idx, int64_t n, bool blurred, std::vector<gpet_event>& out,
                  std::vector<uint8_t>& meta)
{
    out.resize((size_t)n);
    meta.resize((size_t)n);
    if (n == 0) return GPET_OK;
    CK(W.g_ev.ensure((size_t)n * sizeof(EventRec)));
    CK(W.g_meta.ensure((size_t)n));
    PulseDev P = pulse_view(W);
    if (gather_events(P, d_idx, n, blurred, W.dg, W.g_ev.as<EventRec>(), W.g_meta.as<uint8_t>(), c->stream))
        return fail(c, GPET_ERR_CUDA, "gather of event records failed");
    CK(cudaMemcpyAsync(out.data(), W.g_ev.p, (size_t)n * sizeof(EventRec), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(meta.data(), W.g_meta.p, (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return GPET_OK;
}

static bool results(gpet_ctx* c) { return c->have_results && c->work; }

// the device address of pinned (page-locked, mapped) host memory, or null for
// any other memory (pageable, device, unknown)
static void* mapped_host(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" {

int gpet_get_singles(gpet_ctx* c, gpet_event* buf, uint8_t* scat, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    const int64_t off = W.s_off[c->res_sim];
    *n = W.s_off[c->res_sim + 1] - off;
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the singles");
    PulseDev P = pulse_view(W);
    // into pinned caller memory the gather kernel stores the records itself
    // (whole 16-byte words across the host link, no staging copy)
    void* dbuf = mapped_host(buf);
    void* dscat = mapped_host(scat);
    if (dbuf && !(reinterpret_cast<uintptr_t>(dbuf) & 15) && (!scat || dscat)) {
        if (gather_events_mapped(P, W.dg.single_idx + off, *n, W.dg, static_cast<EventRec*>(dbuf),
                                 static_cast<uint8_t*>(dscat), c->stream))
            return fail(c, GPET_ERR_CUDA, "gather of event records failed");
        CK(cudaStreamSynchronize(c->stream));
        return GPET_OK;
    }
    // otherwise gathered on the device and copied into the caller's buffers
    CK(W.g_ev.ensure((size_t)*n * sizeof(EventRec)));
    CK(W.g_meta.ensure((size_t)*n));
    if (gather_events(P, W.dg.single_idx + off, *n, true, W.dg, W.g_ev.as<EventRec>(), W.g_meta.as<uint8_t>(),
                      c->stream))
        return fail(c, GPET_ERR_CUDA, "gather of event records failed");
    CK(cudaMemcpyAsync(buf, W.g_ev.p, (size_t)*n * sizeof(EventRec), cudaMemcpyDeviceToHost, c->stream));
    if (scat) {
        const int64_t blocks = std::min<int64_t>((*n + 255) / 256, 152 * 16);
        k_scat_flags<<<(unsigned)blocks, 256, 0, c->stream>>>(W.g_meta.as<uint8_t>(), *n);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(scat, W.g_meta.p, (size_t)*n, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return GPET_OK;
}

// staging buffer b of group g holding at least n bytes (a growth takes a
// quarter more, so that runs of slightly varying size do not reallocate, and
// first waits for the copies in flight, which may still read the old buffer)
static cudaError_t stage_ensure(gpet_ctx* c, Staged& g, DevBuf& b, size_t n)
{
    if (n <= b.bytes && b.p) return cudaSuccess;
    if (g.pending) {
        cudaError_t e = cudaStreamSynchronize(c->cstream);
        if (e != cudaSuccess) return e;
        c->st_singles.pending = c->st_coinc.pending = false;
    }
    return b.ensure(n + n / 4);
}

// blocks of the kernels of the asynchronous copies: they run beside the next
// run's kernels and are bound by the host link, not by the SMs
constexpr unsigned kCopyBlocks = 64;

// the copy stream starts after everything enqueued on the main stream so far
// (the run whose results are copied)
static cudaError_t copies_after_main(gpet_ctx* c)
{
    cudaError_t e = cudaEventRecord(c->cready, c->stream);
    return e == cudaSuccess ? cudaStreamWaitEvent(c->cstream, c->cready, 0) : e;
}

int gpet_get_singles_async(gpet_ctx* c, gpet_event* buf, uint8_t* scat, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    const int64_t off = W.s_off[c->res_sim];
    *n = W.s_off[c->res_sim + 1] - off;
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the singles");
    Staged& g = c->st_singles;
    const PulseDev P = pulse_view(W);
    void* dbuf = mapped_host(buf);
    void* dscat = mapped_host(scat);
    CK(copies_after_main(c));
    if (dbuf && !(reinterpret_cast<uintptr_t>(dbuf) & 15) && (!scat || dscat)) {
        // pinned caller memory: the tile-staged gather stores the records there
        // itself, across the host link, on the copy stream
        if (gather_events_mapped(P, W.dg.single_idx + off, *n, W.dg, static_cast<EventRec*>(dbuf),
                                 static_cast<uint8_t*>(dscat), c->cstream, kCopyBlocks))
            return fail(c, GPET_ERR_CUDA, "gather of event records failed");
    } else {
        // otherwise gathered into the context's device buffers and copied
        CK(stage_ensure(c, g, g.a, (size_t)*n * sizeof(EventRec)));
        CK(stage_ensure(c, g, g.b, (size_t)*n));
        if (gather_events_mapped(P, W.dg.single_idx + off, *n, W.dg, g.a.as<EventRec>(),
                                 scat ? g.b.as<uint8_t>() : nullptr, c->cstream, kCopyBlocks))
            return fail(c, GPET_ERR_CUDA, "gather of event records failed");
        CK(cudaMemcpyAsync(buf, g.a.p, (size_t)*n * sizeof(EventRec), cudaMemcpyDeviceToHost, c->cstream));
        if (scat) CK(cudaMemcpyAsync(scat, g.b.p, (size_t)*n, cudaMemcpyDeviceToHost, c->cstream));
    }
    CK(cudaEventRecord(g.done, c->cstream));
    g.pending = true;
    return GPET_OK;
}

int gpet_get_coincidences_async(gpet_ctx* c, int64_t* pairs, uint8_t* klass, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    const int64_t off = W.c_off[c->res_sim];
    *n = W.c_off[c->res_sim + 1] - off;
    if (!pairs || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the coincidences");
    Staged& g = c->st_coinc;
    void* dpairs = mapped_host(pairs);
    void* dcls = mapped_host(klass);
    const bool direct = dpairs && (!klass || dcls);
    if (!direct) {
        CK(stage_ensure(c, g, g.a, sizeof(int64_t) * 2 * (size_t)*n));
        CK(stage_ensure(c, g, g.b, (size_t)*n));
    }
    CK(copies_after_main(c));
    int64_t* dp = direct ? static_cast<int64_t*>(dpairs) : g.a.as<int64_t>();
    uint8_t* dc = klass ? (direct ? static_cast<uint8_t*>(dcls) : g.b.as<uint8_t>()) : nullptr;
    const int64_t blocks = std::min<int64_t>((*n + 255) / 256, kCopyBlocks);
    k_coinc_out<<<(unsigned)blocks, 256, 0, c->cstream>>>(W.dg.coinc_pairs + 2 * off, W.dg.coinc_class + off, *n,
                                                          W.s_off[c->res_sim], dp, dc);
    CK(cudaGetLastError());
    if (!direct) {
        CK(cudaMemcpyAsync(pairs, g.a.p, sizeof(int64_t) * 2 * (size_t)*n, cudaMemcpyDeviceToHost, c->cstream));
        if (klass) CK(cudaMemcpyAsync(klass, g.b.p, (size_t)*n, cudaMemcpyDeviceToHost, c->cstream));
    }
    CK(cudaEventRecord(g.done, c->cstream));
    g.pending = true;
    return GPET_OK;
}

int gpet_wait_copies(gpet_ctx* c)
{
    if (!c) return GPET_ERR_ARG;
    if (!c->st_singles.pending && !c->st_coinc.pending) return GPET_OK;
    CK(cudaStreamSynchronize(c->cstream));
    c->st_singles.pending = c->st_coinc.pending = false;
    return GPET_OK;
}

// pulses (or hits) of this context's simulation: indices into the batch buffer
static int own_rows(gpet_ctx* c, Work& W, const DevBuf& simbuf, int64_t total, std::vector<int64_t>& rows)
{
    rows.clear();
    if (W.nsims <= 1) {
        rows.resize((size_t)total);
        for (int64_t i = 0; i < total; ++i) rows[i] = i;
        return GPET_OK;
    }
    std::vector<int32_t> sim((size_t)total);
    if (total) CK(cudaMemcpy(sim.data(), simbuf.p, (size_t)total * 4, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < total; ++i)
        if (sim[i] == c->res_sim) rows.push_back(i);
    return GPET_OK;
}

int gpet_get_pulses(gpet_ctx* c, gpet_event* buf, uint8_t* scat, uint8_t* slot, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    *n = W.nsims <= 1 ? W.n_pulses : (int64_t)W.hcnt[c->res_sim].n_pulse;
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the pulses");
    std::vector<gpet_event> ev;
    std::vector<uint8_t> m;
    int rc = gather(c, W, nullptr, W.n_pulses, false, ev, m);
    if (rc) return rc;
    std::vector<int64_t> rows;
    if ((rc = own_rows(c, W, W.p_sim, W.n_pulses, rows))) return rc;
    std::sort(rows.begin(), rows.end(), [&](int64_t a, int64_t b) {
        if (ev[a].parn != ev[b].parn) return ev[a].parn < ev[b].parn;
        return (m[a] & 0x7f) < (m[b] & 0x7f);
    });
    if ((int64_t)rows.size() != *n) return fail(c, GPET_ERR_CUDA, "pulse counts are inconsistent");
    for (int64_t i = 0; i < *n; ++i) {
        buf[i] = ev[rows[i]];
        if (scat) scat[i] = (m[rows[i]] & 0x80) ? 1 : 0;
        if (slot) slot[i] = m[rows[i]] & 0x7f;
    }
    return GPET_OK;
}

int gpet_get_coincidences(gpet_ctx* c, int64_t* pairs, uint8_t* klass, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    const int64_t off = W.c_off[c->res_sim];
    *n = W.c_off[c->res_sim + 1] - off;
    if (!pairs || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the coincidences");
    CK(cudaMemcpyAsync(pairs, W.dg.coinc_pairs + 2 * off, sizeof(int64_t) * 2 * (size_t)*n, cudaMemcpyDeviceToHost,
                       c->stream));
    if (klass) CK(cudaMemcpyAsync(klass, W.dg.coinc_class + off, (size_t)*n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const int64_t soff = W.s_off[c->res_sim];
    for (int64_t i = 0; i < 2 * *n; ++i) pairs[i] -= soff;
    return GPET_OK;
}

int gpet_get_hits(gpet_ctx* c, int32_t* ids, float* f, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    Work& W = *c->work;
    *n = W.nsims <= 1 ? W.n_hits : (int64_t)W.hcnt[c->res_sim].n_hit;
    if (W.n_hits == 0 || !W.sim_hits[c->res_sim]) *n = 0;
    if ((!ids && !f) || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the hits");
    std::vector<int32_t> hid((size_t)W.n_hits * 5);
    std::vector<float> hf((size_t)W.n_hits * 5);
    CK(cudaMemcpyAsync(hid.data(), W.h_id.p, (size_t)W.n_hits * 20, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hf.data(), W.h_f.p, (size_t)W.n_hits * 20, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::vector<int64_t> rows;
    int rc = own_rows(c, W, W.h_sim, W.n_hits, rows);
    if (rc) return rc;
    if ((int64_t)rows.size() != *n) return fail(c, GPET_ERR_CUDA, "hit counts are inconsistent");
    for (int64_t i = 0; i < *n; ++i) {
        if (ids) std::memcpy(ids + 5 * i, hid.data() + 5 * rows[i], 20);
        if (f) std::memcpy(f + 5 * i, hf.data() + 5 * rows[i], 20);
    }
    return GPET_OK;
}

int gpet_get_exits(gpet_ctx* c, void* buf, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    *n = results(c) ? (int64_t)c->host_exits.size() : 0;
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the exits");
    std::memcpy(buf, c->host_exits.data(), sizeof(ExitRec) * (size_t)*n);
    return GPET_OK;
}

static_assert(sizeof(gpet_psf_record) == sizeof(SrcRec), "phase-space record layouts agree");

// getDistance, gPET_kernals.cu:148-171: distance along u from x to the
// record sphere (centre c, radius r); the root choice is the reference's
static float sphere_distance(const float x[3], const float u[3], const float sph[4])
{
    const float cx = x[0] - sph[0], cy = x[1] - sph[1], cz = x[2] - sph[2];
    const float a = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const float b = 2.0f * (u[0] * cx + u[1] * cy + u[2] * cz);
    const float cc = (cx * cx + cy * cy + cz * cz) - sph[3] * sph[3];
    const float disc = b * b - 4.0f * a * cc;
    if (disc < 0.0f) return 0.0f;
    if (cc < 0.0f) return (-b + std::sqrt(disc)) / (2.0f * a);
    if (b < 0.0f) return (-b - std::sqrt(disc)) / (2.0f * a);
    return (-b + std::sqrt(disc)) / (2.0f * a);
}

// phantom phase space (gPET.cu:91-114, 328-352): photons that left the
// phantom (time > 0), optionally moved onto the record sphere
static void phantom_records(const gpet_ctx* c, std::vector<SrcRec>& out)
{
    out.clear();
    const float* sph = c->cfg.recordsphere;
    for (size_t i = 0; i < c->host_exits.size(); ++i) {
        const ExitRec& e = c->host_exits[i];
        if (e.status != 1 || !(e.t > 0.0)) continue;
        SrcRec r;
        r.x = e.x; r.y = e.y; r.z = e.z; r.ux = e.ux; r.uy = e.uy; r.uz = e.uz; r.E = e.E;
        r.eventid = (int32_t)(i / 2);
        r.t = e.t;
        if (c->psf_sphere) {
            const float x[3] = {e.x, e.y, e.z}, u[3] = {e.ux, e.uy, e.uz};
            const float d = sphere_distance(x, u, sph);
            r.x = e.x + d * e.ux; r.y = e.y + d * e.uy; r.z = e.z + d * e.uz;
            r.t = e.t + (double)d / kSpe;
        }
        out.push_back(r);
    }
}

static void source_records(const gpet_ctx* c, std::vector<SrcRec>& out)
{
    out.clear();
    for (const SrcRec& r : c->host_source)
        if (r.t > 0.0) out.push_back(r);
}

static int append_file(gpet_ctx* c, const std::string& path, const void* p, size_t bytes)
{
    FILE* f = std::fopen(path.c_str(), "ab");
    if (!f) return fail(c, GPET_ERR_IO, "cannot open " + path);
    if (bytes && std::fwrite(p, 1, bytes, f) != bytes) { std::fclose(f); return fail(c, GPET_ERR_IO, "short write " + path); }
    std::fclose(f);
    return GPET_OK;
}

int gpet_write_outputs(gpet_ctx* c, const char* dir)
{
    if (!c || !dir) return GPET_ERR_ARG;
    if (!results(c)) return fail(c, GPET_ERR_ARG, "no results to write");
    std::string d(dir);
    // the directory and its parents are made when missing
    for (size_t i = 1; i <= d.size(); ++i) {
        if (i < d.size() && d[i] != '/') continue;
        const std::string part = d.substr(0, i);
        if (mkdir(part.c_str(), 0755) != 0 && errno != EEXIST)
            return fail(c, GPET_ERR_IO, "cannot make the output directory " + part);
    }
    int64_t n = 0;
    int rc;
    // adder.dat: pulses after adder + readout (gPET.cu:383)
    gpet_get_pulses(c, nullptr, nullptr, nullptr, 0, &n);
    std::vector<gpet_event> ev((size_t)n);
    if (n && (rc = gpet_get_pulses(c, ev.data(), nullptr, nullptr, n, &n))) return rc;
    if ((rc = append_file(c, d + "/adder.dat", ev.data(), sizeof(gpet_event) * (size_t)n))) return rc;
    // HitsID.dat / Hits.dat (gPET.cu:367-379)
    gpet_get_hits(c, nullptr, nullptr, 0, &n);
    std::vector<int32_t> hid((size_t)n * 5);
    std::vector<float> hf((size_t)n * 5);
    if (n && (rc = gpet_get_hits(c, hid.data(), hf.data(), n, &n))) return rc;
    if ((rc = append_file(c, d + "/HitsID.dat", hid.data(), hid.size() * 4))) return rc;
    if ((rc = append_file(c, d + "/Hits.dat", hf.data(), hf.size() * 4))) return rc;
    // singles.dat (gPET.cu:424)
    gpet_get_singles(c, nullptr, nullptr, 0, &n);
    std::vector<gpet_event> sg((size_t)n);
    if (n && (rc = gpet_get_singles(c, sg.data(), nullptr, n, &n))) return rc;
    if ((rc = append_file(c, d + "/singles.dat", sg.data(), sizeof(gpet_event) * (size_t)n))) return rc;
    // coincidences.dat: pairs of Event records; coincidences_class.dat: class bytes
    int64_t nc = 0;
    gpet_get_coincidences(c, nullptr, nullptr, 0, &nc);
    std::vector<int64_t> pr((size_t)nc * 2);
    std::vector<uint8_t> cl((size_t)nc);
    if (nc && (rc = gpet_get_coincidences(c, pr.data(), cl.data(), nc, &nc))) return rc;
    std::vector<gpet_event> ce((size_t)nc * 2);
    for (int64_t i = 0; i < nc; ++i) { ce[2 * i] = sg[pr[2 * i]]; ce[2 * i + 1] = sg[pr[2 * i + 1]]; }
    if ((rc = append_file(c, d + "/coincidences.dat", ce.data(), sizeof(gpet_event) * ce.size()))) return rc;
    if ((rc = append_file(c, d + "/coincidences_class.dat", cl.data(), cl.size()))) return rc;
    // phase-space records: 28-byte state (float3 position, float4 direction +
    // energy), int32 event id, double time in three files each
    auto write_psf = [&](const std::vector<SrcRec>& v, const std::string& stem) -> int {
        std::vector<float> st(v.size() * 7);
        std::vector<int32_t> id(v.size());
        std::vector<double> tt(v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            const SrcRec& r = v[i];
            const float f[7] = {r.x, r.y, r.z, r.ux, r.uy, r.uz, r.E};
            std::memcpy(&st[7 * i], f, sizeof(f));
            id[i] = r.eventid;
            tt[i] = r.t;
        }
        int r2;
        if ((r2 = append_file(c, d + "/out" + stem + ".dat", st.data(), st.size() * 4))) return r2;
        if ((r2 = append_file(c, d + "/id" + stem + ".dat", id.data(), id.size() * 4))) return r2;
        return append_file(c, d + "/time" + stem + ".dat", tt.data(), tt.size() * 8);
    };
    std::vector<SrcRec> v;
    if (!c->host_source.empty()) {
        source_records(c, v);
        if ((rc = write_psf(v, "source"))) return rc;
    }
    if (!c->host_exits.empty()) {
        phantom_records(c, v);
        if ((rc = write_psf(v, "phantom"))) return rc;
    }
    return GPET_OK;
}

int gpet_sinogram(gpet_ctx* c, const gpet_sino_params* sp, uint32_t* out)
{
    if (!c || !sp || !out) return GPET_ERR_ARG;
    if (sp->n_s < 1 || sp->n_phi < 1 || sp->n_z < 1 || !(sp->s_max > 0.0f) || !(sp->z_max > 0.0f) ||
        (int64_t)sp->n_s * sp->n_phi * sp->n_z > (1ll << 31))
        return fail(c, GPET_ERR_ARG, "bad sinogram size");
    const size_t nbins = (size_t)sp->n_s * sp->n_phi * sp->n_z;
    std::memset(out, 0, nbins * 4);
    if (!results(c)) return GPET_OK;
    CK(cudaSetDevice(c->device));
    Work& W = *c->work;
    const int64_t c0 = W.c_off[c->res_sim], nc = W.c_off[c->res_sim + 1] - c0;
    if (nc == 0) return GPET_OK;
    // panel id -> panel record
    std::vector<int32_t> id2p(kMaxPanels, -1);
    for (int i = 0; i < c->geo.npanels; ++i) {
        const int id = (int)c->geo.panels[(size_t)i * kPanelStride + 30];
        if (id >= 0 && id < kMaxPanels) id2p[id] = i;
    }
    DevBuf hist, map;
    CK(hist.ensure(nbins * 4));
    CK(map.ensure(id2p.size() * 4));
    CK(cudaMemsetAsync(hist.p, 0, nbins * 4, c->stream));
    CK(cudaMemcpyAsync(map.p, id2p.data(), id2p.size() * 4, cudaMemcpyHostToDevice, c->stream));
    SinoParams p{sp->n_s, sp->n_phi, sp->n_z, sp->s_max, sp->z_max, sp->class_mask};
    PulseDev P = pulse_view(W);
    if (sinogram_device(W.dg.coinc_pairs, W.dg.coinc_class, c0, nc, W.dg.single_idx, W.dg, P.pann,
                        c->d_panels.as<float>(), map.as<int32_t>(), kMaxPanels, p, hist.as<uint32_t>(), c->stream))
        return fail(c, GPET_ERR_CUDA, "sinogram kernel failed");
    CK(cudaMemcpyAsync(out, hist.p, nbins * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return GPET_OK;
}

int gpet_get_source_records(gpet_ctx* c, gpet_psf_record* buf, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    std::vector<SrcRec> v;
    source_records(c, v);
    *n = (int64_t)v.size();
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the source records");
    std::memcpy(buf, v.data(), sizeof(SrcRec) * v.size());
    return GPET_OK;
}

int gpet_get_phantom_records(gpet_ctx* c, gpet_psf_record* buf, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    if (!results(c)) { *n = 0; return GPET_OK; }
    std::vector<SrcRec> v;
    phantom_records(c, v);
    *n = (int64_t)v.size();
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the phantom records");
    std::memcpy(buf, v.data(), sizeof(SrcRec) * v.size());
    return GPET_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- surrogate glue
namespace gpet {

int ctx_geometry(const gpet_ctx* c, SurGeom* g)
{
    if (!c || !c->have_geo || c->geo.panels.empty()) return GPET_ERR_ARG;
    std::memset(g, 0, sizeof(*g));
    g->device = c->device;
    g->npanels = c->geo.npanels;
    for (int k = 0; k < 15; ++k) g->panel0[k] = c->geo.panels[k];
    g->dirsign = c->geo.panels[18] < 0.0f ? -1.0f : 1.0f;
    g->moduleN = c->geo.moduleN;
    g->crystalN = c->geo.crystalN;
    g->crystalNy = c->geo.crystalNy;
    g->rdepth = c->have_cfg ? c->cfg.rdepth : 2;
    g->rpolicy = c->have_cfg ? c->cfg.rpolicy : 1;
    g->ndetmat = c->geo.ndetmat;
    for (int k = 0; k < c->geo.ndetmat; ++k) { g->det_mat[k] = c->geo.det_mat[k]; g->det_den[k] = c->geo.det_den[k]; }
    return GPET_OK;
}

}  // namespace gpet

extern "C" {

int gpet_set_surrogate(gpet_ctx* c, gpet_surrogate* s)
{
    if (!c) return GPET_ERR_ARG;
    if (s) {
        SurGeom g{};
        if (ctx_geometry(c, &g)) return fail(c, GPET_ERR_ARG, "load the geometry before attaching a surrogate");
        SurrogateDev d{};
        const char* why = "";
        if (surrogate_view(s, g, &d, &why)) return fail(c, GPET_ERR_ARG, why);
    }
    c->sur = s;
    return GPET_OK;
}

int gpet_get_entries(gpet_ctx* c, gpet_entry* buf, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    *n = (int64_t)c->host_entries.size();
    if (!buf || *n == 0) return GPET_OK;
    if (cap < *n) return fail(c, GPET_ERR_ARG, "buffer too small for the entry records");
    std::memcpy(buf, c->host_entries.data(), sizeof(EntryRec) * (size_t)*n);
    return GPET_OK;
}

}  // extern "C"

extern "C" {

// ---------------------------------------------------------------- introspection
int gpet_get_panels(gpet_ctx* c, float* out, int32_t cap, int32_t* np)
{
    if (!c || !np) return GPET_ERR_ARG;
    *np = c->geo.npanels;
    if (!out) return GPET_OK;
    if (cap < *np) return fail(c, GPET_ERR_ARG, "buffer too small for the panels");
    std::memcpy(out, c->geo.panels.data(), sizeof(float) * 32 * (size_t)*np);
    return GPET_OK;
}

int gpet_get_counts(gpet_ctx* c, int32_t out[4])
{
    if (!c || !out) return GPET_ERR_ARG;
    out[0] = c->geo.moduleNy; out[1] = c->geo.moduleN; out[2] = c->geo.crystalNy; out[3] = c->geo.crystalN;
    return GPET_OK;
}

int gpet_get_source_layout(gpet_ctx* c, int64_t* first, int64_t* count, int32_t cap, int32_t* nsrc)
{
    if (!c || !nsrc) return GPET_ERR_ARG;
    if (c->use_psf) { *nsrc = 0; return GPET_OK; }
    std::string e = source_layout(c);
    if (!e.empty()) return fail(c, GPET_ERR_ARG, e);
    *nsrc = (int32_t)c->src_first.size();
    if (!first || !count) return GPET_OK;
    if (cap < *nsrc) return fail(c, GPET_ERR_ARG, "buffer too small for the source layout");
    for (int i = 0; i < *nsrc; ++i) { first[i] = c->src_first[i]; count[i] = c->src_count[i]; }
    return GPET_OK;
}

int gpet_get_majorant(gpet_ctx* c, int which, float* tab, float* e0, float* ide)
{
    if (!c || !tab) return GPET_ERR_ARG;
    const std::vector<float>& w = which == 0 ? c->wck_ph : c->wck_det;
    if (w.size() != (size_t)kNwck) return fail(c, GPET_ERR_ARG, "majorant not built yet");
    std::memcpy(tab, w.data(), 4 * kNwck);
    if (e0) *e0 = c->wck_e0;
    if (ide) *ide = c->wck_ide;
    return GPET_OK;
}

int gpet_get_table(gpet_ctx* c, int which, float* out, int64_t cap, int64_t* n)
{
    if (!c || !n) return GPET_ERR_ARG;
    const std::vector<float>* v = nullptr;
    switch (which) {
    case 0: v = &c->tab.lamph; break;
    case 1: v = &c->tab.compt; break;
    case 2: v = &c->tab.phote; break;
    case 3: v = &c->tab.rayle; break;
    case 4: v = &c->tab.cmpsf; break;
    case 5: v = &c->tab.rayff; break;
    default: return GPET_ERR_ARG;
    }
    *n = (int64_t)v->size();
    if (!out) return GPET_OK;
    if (cap < *n) return GPET_ERR_ARG;
    std::memcpy(out, v->data(), 4 * (size_t)*n);
    return GPET_OK;
}

}  // extern "C"
