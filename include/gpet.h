/* gpet.h - C ABI of libgpet, the GB300-native gPET hot path.
 *
 * The reference exposes no library API: its boundary is the process
 * `./gPET input_PET.in` (main.cu:26-33) reading gPET's input files and writing
 * its output records, and internally the two drivers
 *     void sampleParticle(Source, Isotopes, float tstart, float tend, int nPanels)   gPET.h:155
 *     void simulateParticle(Particle, int ptype, int nPanels)                         gPET.h:154
 * that run on process-global device state set up by loadPhantom/init/
 * read_file_ro/iniPanel/iniwck (gPET.h:129-160). This header replaces that
 * seam with re-entrant calls on an opaque context: plain pointers and sizes,
 * int status returns (0 = success), no global state, one CUDA stream per
 * context. Each entry point names the reference code it replaces.
 *
 * Units as in the reference: energy eV, length cm, time microseconds. */
#ifndef GPET_H
#define GPET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPET_OK 0
#define GPET_ERR_ARG -1       /* bad argument or state */
#define GPET_ERR_IO -2        /* missing or malformed input file */
#define GPET_ERR_CUDA -3      /* CUDA runtime error */
#define GPET_ERR_CAPACITY -4  /* a bounded buffer overflowed; see gpet_last_error */
#define GPET_ERR_NOGPU -5     /* no CUDA device, or the kernels were not built for it */

typedef struct gpet_ctx gpet_ctx;

/* Event record of the reference (gPET.h:87-92): 48 bytes, t at offset 24.
 * singles.dat / adder.dat are arrays of this record (detector.cu:287-307). */
typedef struct {
    int32_t parn, pann, modn, cryn, siten, eventid;
    double t;
    float E, x, y, z;
} gpet_event;

/* Panel record: 32 floats per panel, in this order (object_t, gPET.h:54-78):
 * 0-2 length xyz, 3-5 module size, 6-8 module space, 9-11 crystal size,
 * 12-14 crystal space, 15-17 offset, 18-20 expansion direction, 21-23 local x
 * axis, 24-26 local y axis, 27-29 local z axis, 30 panel id, 31 unused. */
#define GPET_PANEL_STRIDE 32

typedef struct {
    int64_t n_decays;     /* decays simulated */
    int64_t n_pairs;      /* annihilation pairs emitted (beta+ branch) */
    int64_t n_entered;    /* photons that entered a detector panel */
    int64_t n_pulses;     /* pulses after the per-photon adder and readout */
    int64_t n_hits;       /* energy deposits in crystals */
    int64_t n_threshold;  /* pulses after blur and the threshold window */
    int64_t n_deadtime;   /* after dead time */
    int64_t n_singles;    /* after the energy window */
    int64_t n_coinc, n_true, n_scatter, n_random, n_multiple;
    int64_t n_overflow;   /* photons whose pulse or hit list overflowed */
    int64_t n_stepcap;    /* histories stopped by the step cap */
    double ms_total;             /* device time of the whole run (CUDA events) */
    double ms_source_phantom;    /* source + phantom transport kernels */
    double ms_detector;          /* detector transport kernels */
    double ms_digitizer;         /* blur .. energy window, incl. sorts */
    double ms_coincidence;       /* coincidence sorter */
    int64_t kernel_launches;     /* kernels launched by this run */
    int64_t phantom_steps;       /* Woodcock steps in the phantom (all photons) */
    int64_t detector_steps;      /* Woodcock steps in the panels */
    double ms_source;            /* source stage alone (part of ms_source_phantom) */
    double ms_phantom;           /* phantom stage alone (part of ms_source_phantom) */
    int64_t n_surrogate;         /* photons whose detector response came from the surrogate */
    double ms_surrogate;         /* surrogate stage (part of ms_detector) */
    int64_t n_noise;             /* background singles added before the digitizer */
} gpet_run_stats;

/* ------------------------------------------------------------ lifetime */
/* Create a context on CUDA device `device` (iniDevice, iniDevice.cu:1-60). */
int gpet_create(int device, gpet_ctx** out);
void gpet_destroy(gpet_ctx* ctx);
/* Message of the last failing call on this context (never NULL). */
const char* gpet_last_error(gpet_ctx* ctx);

/* Options the reference has no input key for (key=value):
 *   seed (uint64, default 20261203), sim_id, n_decays (exact decay count,
 *   split over sources in proportion to their expected decays),
 *   coinc_window_ns (4), coinc_policy (0 single window with exactly two
 *   singles, 1 all pairs), record_hits (1), record_exits (0),
 *   base_dir (directory relative paths in input_PET.in resolve against),
 *   data_dir (table directory, default <base_dir>/data); launch shape
 *   (results do not depend on it): sub_decays, chunk_decays,
 *   phantom_blocks_per_sm, drain_period, detector_threads, source_threads,
 *   use_graphs (1: each chunk's wave launches replay as one CUDA graph),
 *   autotune (1: gpet_autotune on the first gpet_run), voxel_palette (read
 *   by gpet_set_phantom: 1 (default) stores the phantom as 16-bit indices
 *   into a palette of its distinct (density, material) pairs, 0 as 8-byte
 *   pairs; more distinct pairs than the palette holds (about 32k or more)
 *   fall back to pairs); background singles
 *   (addnoise, gPET_kernals.cu:699-735): noise_lambda_us (mean gap, 0 = off),
 *   noise_emean_ev, noise_sigma_ev, noise_interval_us (1000; each interval
 *   has its own random stream). */
int gpet_set_option(gpet_ctx* ctx, const char* key, const char* value);

/* ------------------------------------------------------------ inputs */
/* Parse input_PET.in (main.cu:50-182) and load everything it references:
 * tables (init, initialize.cu:886-917), phantom (loadPhantom :32-74),
 * detector (read_file_ro detector.cu:64-285, iniPanel initialize.cu:969),
 * and the voxel source (loadIsotopes/readSource :10-31, :116-144) or the
 * PSF (readParticle :76-115). */
int gpet_load_config(gpet_ctx* ctx, const char* input_pet_in);
/* data/input4gPET.{matter,lamph,compt,cmpsf,phote,rayle,rayff} + isotopes.txt
 * (rmater..rrayff, initialize.cu:279-748; loadIsotopes :10-31). */
int gpet_load_tables(gpet_ctx* ctx, const char* data_dir);
/* Voxel phantom from caller buffers (copied): int32 material, float32
 * density, x fastest (loadPhantom + initPhantom, initialize.cu:32-74, 831-884).
 * At most 2^31 - 1 voxels (GPET_ERR_ARG beyond). The upload also builds, on
 * the device, the map of uniform-density neighbourhoods that lets the
 * positron range skip its voxel walk where the density does not change
 * (about 0.1 ms for 128^3 voxels); results do not depend on it. */
int gpet_set_phantom(gpet_ctx* ctx, const int32_t* mat, const float* den, const int32_t dims[3],
                     const float offset[3], const float size[3]);
/* Panel ring from a .geo file (read_file_ro detector.cu:64-285; iniPanel and
 * iniwck for the detector, initialize.cu:919-1224). */
int gpet_load_geometry(gpet_ctx* ctx, const char* geo_path);
/* source.txt (readSource, initialize.cu:116-144) for the window [tstart, tend] s. */
int gpet_set_source_file(gpet_ctx* ctx, const char* source_txt, float tstart, float tend);
/* Phase-space source from caller buffers: n records of 8 doubles
 * x,y,z,t,vx,vy,vz,E; ptype 0 positron, 1 photon (readParticle,
 * initialize.cu:76-115; simulateParticle gPET.cu:13-199). */
int gpet_set_source_psf(gpet_ctx* ctx, const double* rec8, int64_t n, int ptype);

/* ------------------------------------------------------------ run */
/* Simulate the configured source and digitize: sampleParticle (gPET.cu:201-437)
 * or simulateParticle (gPET.cu:13-199) followed by the coincidence sorter.
 * The previous run's results are dropped when a run starts; a run that fails
 * leaves none (the gpet_get_* calls then report 0 records). */
int gpet_run(gpet_ctx* ctx, gpet_run_stats* stats);
/* No counterpart in the reference (one simulation per process there).
 * Runs n independent simulations (contexts on one device, each fully loaded;
 * each keeps its own tables, phantom, geometry, source, seed and digitizer
 * settings) as one job: their decays are concatenated into shared waves so
 * that many small simulations fill the GPU together, and one digitizer pass
 * sorts all pulses by (simulation, time). Afterwards each context reads its
 * own results with the gpet_get_* calls, identical bit for bit to what
 * gpet_run on that context alone gives. stats[i] (may be NULL) receives each
 * simulation's counts; the timings are those of the whole job. record_exits
 * must be 0 when n > 1. */
int gpet_run_batched(gpet_ctx* const* ctxs, int32_t n, gpet_run_stats* stats);
/* No counterpart in the reference. Launch-shape parameters of the transport
 * (also settable as options): none changes a result, only the time. */
typedef struct {
    int64_t sub_decays;            /* decays per wave (source -> phantom through L2), option sub_decays */
    int64_t chunk_decays;          /* decays per detector pass (queue capacity), option chunk_decays */
    int32_t phantom_blocks_per_sm; /* k_phantom occupancy, option phantom_blocks_per_sm (0 = as many as fit) */
    int32_t drain_period;          /* k_phantom compaction period: staged photons taken through the panel
                                      search once this many (1..32) wait, option drain_period */
    int32_t detector_threads;      /* threads per k_detector block, option detector_threads */
    int32_t source_threads;        /* threads per k_source block, option source_threads */
    int32_t candidates;            /* shapes timed */
    int64_t sample_decays;         /* decays each candidate ran */
    double ms_default, ms_tuned;   /* transport device time of the sample, before and after */
} gpet_tuning;
/* Time candidate shapes on the first sample_decays (<= 0: min(total, 2^24))
 * decays of this context's own workload, coordinate descent over the fields
 * of gpet_tuning, and keep the fastest in the context. Discards the context's
 * previous results. Option autotune=1 runs it on the first gpet_run. */
int gpet_autotune(gpet_ctx* ctx, int64_t sample_decays, gpet_tuning* out);
/* Digitizer + coincidence sorter alone on a caller pulse list (the digitizer
 * chain of gPET.cu:385-424): scat[i] != 0 marks a photon that scattered in the
 * phantom, slot[i] is the pulse's index within its photon's readout list. */
int gpet_digitize(gpet_ctx* ctx, const gpet_event* pulses, const uint8_t* scat, const uint8_t* slot, int64_t n,
                  gpet_run_stats* stats);

/* ------------------------------------------------------------ outputs */
/* Each copies into caller memory; with buf == NULL only *n is set.
 * gpet_get_singles: when buf (16-byte aligned) and scat (or scat == NULL) are
 * pinned host memory, the gather kernel writes the records there itself
 * instead of staging them on the device and copying. */
int gpet_get_singles(gpet_ctx* ctx, gpet_event* buf, uint8_t* scat, int64_t cap, int64_t* n);
/* Pulses after adder + readout, ordered by (parn, slot) (adder.dat content). */
int gpet_get_pulses(gpet_ctx* ctx, gpet_event* buf, uint8_t* scat, uint8_t* slot, int64_t cap, int64_t* n);
/* Coincidences: index pairs into the singles list and class (0 true,
 * 1 scatter, 2 random). */
int gpet_get_coincidences(gpet_ctx* ctx, int64_t* pairs, uint8_t* klass, int64_t cap, int64_t* n);
/* Asynchronous forms of gpet_get_singles / gpet_get_coincidences (the
 * writeSingles / writeCoinc outputs of the reference's main loop, main.cu,
 * for callers that stream acquisitions): the records are gathered on the
 * device (the call waits for that, a fraction of a millisecond) and copied
 * into the caller's buffers on the context's copy stream, which overlaps the
 * context's next gpet_set_phantom / gpet_run. *n is set at once; the buffers
 * (page-locked host memory for the copy to be asynchronous) hold the records
 * only after gpet_wait_copies, and must not be reused or freed before it.
 * Results are identical to the synchronous calls. */
int gpet_get_singles_async(gpet_ctx* ctx, gpet_event* buf, uint8_t* scat, int64_t cap, int64_t* n);
int gpet_get_coincidences_async(gpet_ctx* ctx, int64_t* pairs, uint8_t* klass, int64_t cap, int64_t* n);
/* Waits for the copies of the asynchronous calls above. */
int gpet_wait_copies(gpet_ctx* ctx);
/* Hits (HitsID.dat / Hits.dat records, gPET.cu:367-379): ids [n][5] = parn,
 * panel, module, crystal, type (1/2 Compton, 4 photoelectric); f [n][5] = E,
 * t, local x, y, z. Order within a photon is deposit order. */
int gpet_get_hits(gpet_ctx* ctx, int32_t* ids, float* f, int64_t cap, int64_t* n);
/* Phantom exit state of every photon (option record_exits=1): per photon 12
 * words: x,y,z,ux,uy,uz,E (float), nscat (int32), t (double), status (int32:
 * 0 absorbed, 1 escaped, 2 not emitted, 3 step cap), panel (int32, -1 none). */
int gpet_get_exits(gpet_ctx* ctx, void* buf, int64_t cap, int64_t* n);
/* Phase-space records (OUTPUTPSF 1/2, gPET.cu:63-114, 296-352), 40 bytes:
 * position, direction, energy (float), event id (int32), time (double, us). */
typedef struct {
    float x, y, z, ux, uy, uz, E;
    int32_t eventid;
    double t;
} gpet_psf_record;
/* Emitted photons (option record_source=1): the annihilation photons (or
 * the PSF's photons) as they leave the source stage, time > 0 only. */
int gpet_get_source_records(gpet_ctx* ctx, gpet_psf_record* buf, int64_t cap, int64_t* n);
/* Photons leaving the phantom (option record_exits=1), time > 0 only; with
 * option psf_sphere=1 moved along their direction onto the record sphere of
 * input_PET.in (getDistance, gPET_kernals.cu:148-171; RECORDPSF -1). */
int gpet_get_phantom_records(gpet_ctx* ctx, gpet_psf_record* buf, int64_t cap, int64_t* n);
/* No counterpart in the reference (its list-mode output stops at the
 * singles; readOutput.m reads the records). The last run's coincidences
 * binned into a sinogram by single-slice rebinning: for each pair, the line
 * between the two singles' global positions (their blurred panel-local
 * positions mapped through the panel axes) gives the angle phi in [0, pi),
 * the signed distance s of the line from the z axis and the mean z;
 * out[(iz * n_phi + iphi) * n_s + is] (n_s * n_phi * n_z counts) counts the
 * pairs with s in [-s_max, s_max), z in [-z_max, z_max) whose class bit is in
 * class_mask (1 true, 2 scatter, 4 random). */
typedef struct {
    int32_t n_s, n_phi, n_z;
    float s_max, z_max;           /* cm */
    int32_t class_mask;
} gpet_sino_params;
int gpet_sinogram(gpet_ctx* ctx, const gpet_sino_params* params, uint32_t* out);
/* Append the run's records to out_dir: singles.dat, adder.dat, HitsID.dat,
 * Hits.dat (outevents/outputData, detector.cu:287-307, 387-408) and
 * coincidences.dat (+ coincidences_class.dat); with record_source=1
 * outsource.dat / idsource.dat / timesource.dat, with record_exits=1
 * outphantom.dat / idphantom.dat / timephantom.dat (28-byte state, int32 id,
 * double time per photon, the reference's layouts). out_dir and its parents
 * are made when missing. */
int gpet_write_outputs(gpet_ctx* ctx, const char* out_dir);

/* ------------------------------------------------------------ introspection */
int gpet_get_panels(gpet_ctx* ctx, float* out, int32_t cap, int32_t* npanels);
/* moduleNy, moduleN, crystalNy, crystalN (iniPanel, initialize.cu:1074-1086) */
int gpet_get_counts(gpet_ctx* ctx, int32_t out[4]);
/* decays per source: first index and count */
int gpet_get_source_layout(gpet_ctx* ctx, int64_t* first, int64_t* count, int32_t cap, int32_t* nsrc);
/* Woodcock majorant table (which 0 phantom, 1 detector): 4096 floats + e0, 1/de */
int gpet_get_majorant(gpet_ctx* ctx, int which, float* tab4096, float* e0, float* ide);
/* tables as parsed: which 0 lamph 1 compt 2 phote 3 rayle 4 cmpsf 5 rayff */
int gpet_get_table(gpet_ctx* ctx, int which, float* out, int64_t cap, int64_t* n);

/* ------------------------------------------------------------ allocation-free digitizer */
/* No counterpart in the reference. gpet_digitize_static runs the same
 * digitizer and coincidence sorter as gpet_digitize, but for callers that
 * cannot allocate device memory: code running inside another framework's
 * memory pool or allocator, code whose device allocations are fixed at
 * start-up (real-time acquisition front ends), or code that must not
 * synchronise the device the way cudaMalloc/cudaFree do. It allocates
 * nothing: its working memory is one file-scope device array of
 * GPET_STATIC_ARENA_BYTES, which every GPU that loads the library holds until
 * the process exits, and the caller passes inputs and outputs as device
 * pointers it already owns.
 *
 * Limits and behaviour:
 *  - n <= GPET_STATIC_MAX_PULSES; larger inputs are rejected (GPET_ERR_ARG,
 *    message in err when err != NULL); more singles or pairs than the caller's
 *    capacities -> GPET_ERR_CAPACITY, nothing written past them.
 *  - Every call looks up the array's device address in the CUDA context
 *    current at that moment (the address belongs to the context, not the
 *    device number, so nothing is cached across calls).
 *  - A CUDA error already pending from the caller's earlier work is reported
 *    (GPET_ERR_CUDA) and left pending; a readout slot of 128 or more is
 *    refused with GPET_ERR_ARG, as gpet_digitize refuses it.
 *  - All calls share the one array, which keeps the last call's contents:
 *    calls whose work overlaps on the GPU (two host threads, or two streams of
 *    one device) race and must be serialised by the caller.
 *  - The call enqueues on `stream` (a cudaStream_t; NULL = legacy default) and
 *    synchronises it before returning, because the counts size later steps.
 *  - counts[8] (host) receives: after threshold, after dead time, singles,
 *    coincidences, true, scatter, random, multiples.
 * Inputs: d_pulses[n] (48-byte Event records), d_scat[n] (phantom-scatter
 * flag), d_slot[n] (index within the photon's readout list, < 128).
 * Outputs: d_singles[singles_cap] in time order, d_single_scat, d_pairs
 * [pairs_cap][2] (indices into the singles) and d_class[pairs_cap]. */
#define GPET_STATIC_MAX_PULSES 131072
#define GPET_STATIC_ARENA_BYTES (16u * 1024u * 1024u)

typedef struct {
    int32_t blurpolicy;           /* energy blur, main.cu:171 */
    float Eref, Rref, Eslope, Sblur;
    float Eth;                    /* threshold before dead time, main.cu:166 */
    int32_t dlevel, dtype;        /* dead time level and policy, main.cu:176 */
    float dtime_us;
    float ewin_lo, ewin_hi;       /* energy window, main.cu:181 */
    double coinc_window_ns;
    int32_t coinc_policy;
    int32_t moduleN, crystalN;    /* site numbering of the detector */
    uint64_t seed;
    uint32_t sim_id;
} gpet_digi_params;

int gpet_digitize_static(const gpet_digi_params* prm, const gpet_event* d_pulses, const uint8_t* d_scat,
                         const uint8_t* d_slot, int64_t n, gpet_event* d_singles, uint8_t* d_single_scat,
                         int64_t singles_cap, int64_t* d_pairs, uint8_t* d_class, int64_t pairs_cap,
                         int64_t counts[8], void* stream, char* err, int32_t err_len);

#ifdef __cplusplus
}
#endif
#endif
