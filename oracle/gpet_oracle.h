/* gpet_oracle.h - CPU oracle for the gPET hot path (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle restates, in plain C, the reference gPET algorithm for the path
 * source -> positron range -> annihilation -> Woodcock transport in the voxel
 * phantom -> panel entry -> Woodcock transport in the detector panels ->
 * per-photon adder/readout -> digitizer (blur, threshold, dead time, energy
 * window) -> coincidence sorting. Each function cites the reference file:line
 * it follows. It is the checker of the CUDA implementation and the timed CPU
 * baseline; nothing in the product links or calls it.
 *
 * One source, two builds:
 *   liboracle_fp64.so : transport in double precision with libm (the physics
 *                       oracle: statistical parity target)
 *   liboracle_fp32.so : transport in single precision with the deterministic
 *                       math of detmath.h, operation for operation the same as
 *                       the CUDA kernels (history-level comparison)
 * The digitizer works on the reference's Event record (float E/x/y/z, double t)
 * in both builds, so it is bit-exact against the GPU digitizer on the same
 * pulse list.
 *
 * Parity anchors: the reference ships no tests or golden vectors; the oracle
 * is pinned by known-answer tests derived from the reference's own data files
 * (tables at 511 keV, isotope spectrum, geometry counts, record layouts). */
#ifndef GPET_ORACLE_H
#define GPET_ORACLE_H
#include <stdint.h>

#define OR_PANEL_STRIDE 32
#define OR_MAXSURF 5

/* Event record of the reference, gPET.h:87-92 (48 bytes, t at offset 24) */
typedef struct {
    int32_t parn, pann, modn, cryn, siten, eventid;
    double t;
    float E, x, y, z;
} or_event;

typedef struct {
    /* 1-D cross-section tables on one energy grid (initialize.cu:370-481,
     * 568-662): [nmat][ne] in cm^2/g */
    int32_t nmat, ne;
    float e0, idle;               /* first energy, (ne-1)/(e[ne-1]-e[0]) */
    const float *lamph, *compt, *phote, *rayle;
    /* inverse-CDF surfaces (initialize.cu:483-566, 664-748): [nmat][ncp][nee] */
    int32_t ncp_c, ne_c;  float idcp_c, ide_c;  const float* cmpsf;
    int32_t ncp_r, ne_r;  float idcp_r, ide_r;  const float* rayff;
    float eminph, emax;           /* .matter header: Woodcock grid range */
    /* phantom (initialize.cu:32-74): int32 mat, float32 den, x fastest */
    int32_t nx, ny, nz;
    float dx, dy, dz, offx, offy, offz;
    const int32_t* mat;
    const float* den;
    /* detector (detector.cu:64-285): [npanels][OR_PANEL_STRIDE] floats, see
     * gpet.h for the field order; two materials (crystal, gap) */
    int32_t npanels;
    const float* panels;
    int32_t det_mat[2];
    float det_den[2];
    int32_t moduleN, crystalN, moduleNy, crystalNy;
    int32_t nsurface;
    float surface[10 * OR_MAXSURF];
    /* sources: decay index ranges [first, first+count) per source */
    int32_t nsrc;
    const int64_t *src_first, *src_count;
    const int32_t *src_type, *src_shape;
    const float* src_coef;        /* [nsrc][6] */
    const float *iso_halftime, *iso_ratio, *iso_coef;  /* per isotope type, coef [8] */
    double tstart_s, dt_s;
    int32_t useprange;
    float noncol_sigma, eabsph;
    /* PSF source (initialize.cu:76-115): [npsf][8] doubles x,y,z,t,vx,vy,vz,E;
     * ptype 0 positron, 1 photon. Used when npsf > 0 instead of sources. */
    int64_t npsf;
    const double* psf;
    int32_t psf_ptype;
    /* digitizer (main.cu:158-182) */
    int32_t rdepth, rpolicy, blurpolicy;
    float Eref, Rref, Eslope, Sblur, Eth;
    int32_t dlevel, dtype;
    float dtime_us, ewin_lo, ewin_hi;
    double coinc_window_us;
    int32_t coinc_policy;         /* 0: single window, exactly two; 1: all pairs */
    uint64_t seed;
    uint32_t sim_id;
    /* background singles (addnoise, gPET_kernals.cu:699-735): mean time
     * between them (us, 0 = off), energy mean and spread (eV), the length of
     * the intervals each drawn from its own stream, and the window (us) */
    float noise_lambda_us, noise_emean, noise_sigma;
    double noise_interval_us, noise_t0_us, noise_t1_us;
    /* detector materials beyond the reference's two: crystal regions marked
     * by quadratic surface k are material xdet_mat[k] at xdet_den[k] */
    int32_t nxdet;
    int32_t xdet_mat[6];
    float xdet_den[6];
    /* uniform-density map of the positron range (oracle_build_prmap), or
     * NULL: every positron walks */
    const int8_t* prmap;
} or_scene;

typedef struct {
    float x, y, z, ux, uy, uz, E;
    int32_t nscat;                 /* phantom scatters */
    double t;
    int32_t status;                /* 0 absorbed, 1 escaped, 2 no photon, 3 step cap */
    int32_t panel;                 /* entered panel index, -1 none */
} or_exit;

/* an emitted photon (the source phase space, gPET.cu:63-87): t = 0 when the
 * photon slot carries nothing */
typedef struct {
    float x, y, z, ux, uy, uz, E;
    int32_t eventid;
    double t;
} or_src;

typedef struct {
    int64_t n_decays, n_pairs, n_entered;
    int64_t n_pulses, n_hits;
    int64_t n_threshold, n_deadtime, n_singles;
    int64_t n_coinc, n_true, n_scatter, n_random, n_multiple;
    int64_t n_overflow, n_stepcap, n_noise;
    /* arrays owned by the oracle, free with oracle_free_result */
    or_exit* exits;               /* [2*n_decays] when requested */
    or_src* source;               /* [2*n_decays] when requested */
    or_event* pulses;             /* after adder + readout, sorted by (parn, slot) */
    uint8_t* pulse_scat;
    uint8_t* pulse_slot;
    int32_t* hit_id;              /* [n_hits][5] parn pann modn cryn type */
    float* hit_f;                 /* [n_hits][5] E t x y z */
    or_event* singles;            /* time order */
    uint8_t* single_scat;
    uint8_t* single_slot;
    int64_t* coinc;               /* [n_coinc][2] indices into singles */
    uint8_t* coinc_class;         /* 0 true, 1 scatter, 2 random */
} or_result;

/* Simulate decays [d_begin, d_end) (or PSF records) and digitize.
 * flags bit0: record exits; bit1: record hits; bit2: record the emitted
 * photons. Returns 0 on success. */
int oracle_run(const or_scene* sc, int64_t d_begin, int64_t d_end, int nthreads, int flags, or_result* out);
/* Digitizer + coincidence sorter alone on a given pulse list (same semantics). */
int oracle_digitize(const or_scene* sc, const or_event* pulses, const uint8_t* scat, const uint8_t* slot,
                    int64_t n, or_result* out);
void oracle_free_result(or_result* r);
/* Philox4x32-10 block, for known-answer tests. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The uniforms the samplers make of words w. */
void oracle_u01(int64_t n, const uint32_t* w, float* out);
/* The first n words of the stream (key k0 k1, tag, id): xoshiro128** from the
 * Philox4x32-10 block of counter (0, tag, id), for known-answer tests. */
void oracle_stream_words(uint32_t k0, uint32_t k1, uint32_t tag, uint64_t id, int64_t n, uint32_t* out);
int oracle_real_bytes(void);

#endif
