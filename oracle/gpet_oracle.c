/* gpet_oracle.c - CPU oracle for the gPET hot path. TEST INFRASTRUCTURE ONLY:
 * imported by the tests and by bench.py's CPU-baseline leg, never by the
 * product. See gpet_oracle.h for what it restates and how it is built.
 *
 * Build: ORACLE_FP32 defined -> single-precision transport with detmath.h
 * (operation-for-operation twin of the CUDA kernels); otherwise double
 * precision transport with libm. Compile with -ffp-contract=off. */
#include "gpet_oracle.h"
#include "../gpet_gb300/csrc/detmath.h"

#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_FP32
typedef float real;
#define R_LOG(x) dm_logf(x)
#define R_EXP(x) dm_expf(x)
#define R_SQRT(x) dm_sqrt(x)
#define R_CBRT(x) dm_cbrtf(x)
#define R_FLOOR(x) floorf(x)
#define R_FABS(x) fabsf(x)
#define R_FMA(a, b, c) dm_fma(a, b, c)
static inline void r_sincos_turns(real u, real* s, real* c) { dm_sincos_turns(u, s, c); }
#else
typedef double real;
#define R_LOG(x) log(x)
#define R_EXP(x) exp(x)
#define R_SQRT(x) sqrt(x)
#define R_CBRT(x) cbrt(x)
#define R_FLOOR(x) floor(x)
#define R_FABS(x) fabs(x)
#define R_FMA(a, b, c) fma(a, b, c)
static inline void r_sincos_turns(real u, real* s, real* c)
{
    double a = 6.283185307179586476925 * u;
    *s = sin(a);
    *c = cos(a);
}
#endif

#define C_MC2 ((real)510999.1)          /* constants.h:37 MC2 (eV) */
#define C_IMC2 ((real)1.95695060911e-6) /* constants.h:38 */
#define C_SPE 29979.2458                /* cm/us, gPET_kernals.cu:264 */
/* Flight times: the FP32 build (like the kernels) accumulates a photon's
 * flight time in single precision and adds it to its double-precision time
 * stamp once; the FP64 build accumulates in double at every step, as the
 * reference does (gPET_kernals.cu:283, 1025). */
#ifdef ORACLE_FP32
#define TIME_STEP(p, s) ((p)->tf = dm_fma((s), DM_INV_SPEED, (p)->tf))
#else
#define TIME_STEP(p, s) ((p)->t += (double)(s) / C_SPE)
#endif
#define MAX_STEPS 100000
#define MAX_PULSE 8   /* distinct crystals per photon in the adder list */
#define MAX_HITS 16   /* deposits recorded per photon */

enum { TAG_DECAY = 1, TAG_PHANTOM = 2, TAG_DET = 4, TAG_BLUR = 8, TAG_NOISE = 9 };

/* ------------------------------------------------------------------ RNG */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), restated from the paper. */
void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* A stream (key, tag, 64-bit id): its state is the Philox4x32-10 block of
 * counter (0, tag, id) under the key (the all-zero state, which xoshiro never
 * leaves, replaced by a fixed one); its words come from xoshiro128**
 * (Blackman & Vigna, "Scrambled linear pseudorandom number generators", ACM
 * TOMS 2021), restated from the paper. */
typedef struct {
    uint32_t s[4];
#ifdef ORACLE_TAPE
    const uint32_t* tape;   /* words to draw instead of the stream's (pins against the reference) */
    int64_t tape_n, tape_pos;
#endif
} stream_t;

static void st_seed_words(stream_t* s, uint32_t k0, uint32_t k1, uint32_t tag, uint64_t id)
{
    const uint32_t key[2] = {k0, k1};
    const uint32_t ctr[4] = {0u, tag, (uint32_t)id, (uint32_t)(id >> 32)};
    oracle_philox4x32_10(ctr, key, s->s);
    if ((s->s[0] | s->s[1] | s->s[2] | s->s[3]) == 0u) s->s[0] = 0x9E3779B9u;
#ifdef ORACLE_TAPE
    s->tape = NULL;
#endif
}

static void st_init(stream_t* s, const or_scene* sc, uint32_t tag, uint64_t id)
{
    st_seed_words(s, (uint32_t)sc->seed, (uint32_t)(sc->seed >> 32) + sc->sim_id, tag, id);
}

static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

static inline uint32_t st_next(stream_t* s)
{
#ifdef ORACLE_TAPE
    if (s->tape) {
        const uint32_t w = s->tape_pos < s->tape_n ? s->tape[s->tape_pos] : 0x80000000u;
        s->tape_pos++;
        return w;
    }
#endif
    uint32_t* q = s->s;
    const uint32_t v = rotl32(q[1] * 5u, 7) * 9u;
    const uint32_t t = q[1] << 9;
    q[2] ^= q[0];
    q[3] ^= q[1];
    q[1] ^= q[2];
    q[0] ^= q[3];
    q[2] ^= t;
    q[3] = rotl32(q[3], 11);
    return v;
}

/* uniforms the samplers make of words w (dm_u01), for known-answer tests */
void oracle_u01(int64_t n, const uint32_t* w, float* out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = dm_u01(w[i]);
}

/* the first n words of stream (key, tag, id), for known-answer tests */
void oracle_stream_words(uint32_t k0, uint32_t k1, uint32_t tag, uint64_t id, int64_t n, uint32_t* out)
{
    stream_t s;
    st_seed_words(&s, k0, k1, tag, id);
    for (int64_t i = 0; i < n; ++i) out[i] = st_next(&s);
}

static inline real st_u(stream_t* s) { return (real)dm_u01(st_next(s)); }

static inline double st_ud(stream_t* s)
{
    uint32_t hi = st_next(s);
    uint32_t lo = st_next(s);
    return dm_u01d(hi, lo);
}

/* normal deviate: Box-Muller, two uniforms (replaces curand_normal) */
static inline void st_normal2(stream_t* s, real* n1, real* n2)
{
    real u1 = st_u(s), u2 = st_u(s);
#ifdef ORACLE_FP32
    dm_normal2(u1, u2, n1, n2);
#else
    real sn, cs;
    r_sincos_turns(u2, &sn, &cs);
    real R = R_SQRT((real)-2.0 * R_LOG(u1));
    *n1 = R * cs;
    *n2 = R * sn;
#endif
}

static inline real st_normal(stream_t* s)
{
    real u1 = st_u(s), u2 = st_u(s);
    real sn, cs;
    r_sincos_turns(u2, &sn, &cs);
    return R_SQRT((real)-2.0 * R_LOG(u1)) * cs;
}

/* uniform in float in both builds (digitizer stages) */
static inline float st_uf(stream_t* s) { return dm_u01(st_next(s)); }

/* the digitizer always computes in the Event record's float */
static inline float st_normal_f(stream_t* s)
{
    float u1 = dm_u01(st_next(s)), u2 = dm_u01(st_next(s));
    return dm_normal(u1, u2);
}

int oracle_real_bytes(void) { return (int)sizeof(real); }

/* --------------------------------------------------------------- lookups */
/* linear interpolation at fractional index x with edge clamping: the value the
 * reference's linearly filtered 1-D textures return (gPET_kernals.cu:31-64) */
static inline real lerp1(const float* tab, int n, real x)
{
    if (!(x > (real)0.0)) return (real)tab[0];
    if (x >= (real)(n - 1)) return (real)tab[n - 1];
    int i = (int)x;
    real f = x - (real)i;
    real a = (real)tab[i], b = (real)tab[i + 1];
    return R_FMA(f, b - a, a);
}

/* bilinear lookup of an inverse-CDF surface [ncp][ne] at (energy index xe,
 * probability index ycp), clamped: tex3D(s_tex/f_tex) gPET_kernals.cu:82,142 */
static inline real lerp2(const float* s, int ncp, int ne, real xe, real ycp)
{
    if (!(xe > (real)0.0)) xe = (real)0.0;
    if (xe > (real)(ne - 1)) xe = (real)(ne - 1);
    if (!(ycp > (real)0.0)) ycp = (real)0.0;
    if (ycp > (real)(ncp - 1)) ycp = (real)(ncp - 1);
    int ie = (int)xe; if (ie > ne - 2) ie = ne - 2;
    int ic = (int)ycp; if (ic > ncp - 2) ic = ncp - 2;
    real fe = xe - (real)ie, fc = ycp - (real)ic;
    const float* r0 = s + (size_t)ic * ne;
    const float* r1 = r0 + ne;
    real a = R_FMA(fe, (real)r0[ie + 1] - (real)r0[ie], (real)r0[ie]);
    real b = R_FMA(fe, (real)r1[ie + 1] - (real)r1[ie], (real)r1[ie]);
    return R_FMA(fc, b - a, a);
}

static inline real xs_at(const or_scene* sc, const float* tab, int m, real e)
{
    real x = (real)sc->idle * (e - (real)sc->e0);
    return lerp1(tab + (size_t)m * sc->ne, sc->ne, x);
}

/* Woodcock majorant tables (replaces iniwck, initialize.cu:773-829, 919-966):
 * node i at e_i = eminph + de*i, de = (emax - eminph)/4096 (the reference's
 * (1-1e-10) factor is 1 in float). Each node stores 1/max over materials of
 * rho_max(m) * max(mu_m over [e_{i-1}, e_{i+1}]) of the linearly interpolated
 * table, so the interpolated majorant bounds every material everywhere. */
#define NWCK 4096
typedef struct { float e0, ide; float tab[NWCK]; } wck_t;

static double xs_lerp_d(const or_scene* sc, const float* tab, double e)
{
    double x = (double)sc->idle * (e - (double)sc->e0);
    if (!(x > 0.0)) return tab[0];
    if (x >= sc->ne - 1) return tab[sc->ne - 1];
    int i = (int)x;
    double f = x - i;
    return tab[i] + f * ((double)tab[i + 1] - (double)tab[i]);
}

static void build_wck(const or_scene* sc, const float* maxden, wck_t* w)
{
    float de = (sc->emax - sc->eminph) / (float)NWCK;
    w->e0 = sc->eminph;
    w->ide = 1.0f / de;
    for (int i = 0; i < NWCK; ++i) {
        double lo = (double)sc->eminph + (double)de * (double)(i > 0 ? i - 1 : 0);
        double hi = (double)sc->eminph + (double)de * (double)(i + 1);
        double best = 0.0;
        for (int m = 0; m < sc->nmat; ++m) {
            if (!(maxden[m] > 0.0f)) continue;
            const float* tab = sc->lamph + (size_t)m * sc->ne;
            double mx = xs_lerp_d(sc, tab, lo);
            double v = xs_lerp_d(sc, tab, hi);
            if (v > mx) mx = v;
            double xlo = (double)sc->idle * (lo - (double)sc->e0);
            double xhi = (double)sc->idle * (hi - (double)sc->e0);
            int k0 = (int)ceil(xlo), k1 = (int)floor(xhi);
            if (k0 < 0) k0 = 0;
            if (k1 > sc->ne - 1) k1 = sc->ne - 1;
            for (int k = k0; k <= k1; ++k)
                if (tab[k] > mx) mx = tab[k];
            mx *= (double)maxden[m];
            if (mx > best) best = mx;
        }
        w->tab[i] = (float)(1.0 / best);
    }
}

static inline real wck_at(const wck_t* w, real e)
{
    return lerp1(w->tab, NWCK, (real)w->ide * (e - (real)w->e0));
}

/* -------------------------------------------------------------- geometry */
/* rotate(): gPET_kernals.cu:172-254 (direction change by polar cos and
 * azimuth; the azimuth is given in turns, phi = 2*pi*u) */
static void rotate(real* u, real* v, real* w, real costh, real phi_turns)
{
    real rho2 = (*u) * (*u) + (*v) * (*v);
    real norm = rho2 + (*w) * (*w);
    if (R_FABS(norm - (real)1.0) > (real)1.0e-4) {
        norm = (real)1.0 / R_SQRT(norm);
        *u = (*u) * norm; *v = (*v) * norm; *w = (*w) * norm;
    }
    real sinphi, cosphi;
    r_sincos_turns(phi_turns, &sinphi, &cosphi);
    real temp = costh * costh;
    if (rho2 > (real)1.0e-20f) {
        real sthrho = temp < (real)1.0 ? R_SQRT(((real)1.0 - temp) / rho2) : (real)0.0;
        real urho = (*u) * sthrho, vrho = (*v) * sthrho;
        real uu = (*u) * costh - vrho * sinphi + (*w) * urho * cosphi;
        real vv = (*v) * costh + urho * sinphi + (*w) * vrho * cosphi;
        real ww = (*w) * costh - rho2 * sthrho * cosphi;
        *u = uu; *v = vv; *w = ww;
    } else {
        real sinth = temp < (real)1.0 ? R_SQRT((real)1.0 - temp) : (real)0.0;
        *v = sinth * sinphi;
        if (*w > (real)0.0) { *u = sinth * cosphi; *w = costh; }
        else { *u = -sinth * cosphi; *w = -costh; }
    }
}

/* getAbsVox, gPET_kernals.cu:19-29: index = trunc((x-off)*idx); an index of 0
 * counts as outside (the reference tests `<= 0` on the truncated value), so
 * inside means 1 <= (x-off)*idx < n in every axis. */
static inline int abs_vox(const or_scene* sc, real idx, real idy, real idz,
                          real x, real y, real z, int* ix, int* iy, int* iz)
{
    real vx = (x - (real)sc->offx) * idx;
    real vy = (y - (real)sc->offy) * idy;
    real vz = (z - (real)sc->offz) * idz;
    int in = vx >= (real)1.0 && vx < (real)sc->nx && vy >= (real)1.0 && vy < (real)sc->ny &&
             vz >= (real)1.0 && vz < (real)sc->nz;
    if (in) { *ix = (int)vx; *iy = (int)vy; *iz = (int)vz; }
    return in;
}

static inline float den_clamped(const or_scene* sc, int ix, int iy, int iz)
{
    if (ix < 0) ix = 0; if (ix > sc->nx - 1) ix = sc->nx - 1;
    if (iy < 0) iy = 0; if (iy > sc->ny - 1) iy = sc->ny - 1;
    if (iz < 0) iz = 0; if (iz > sc->nz - 1) iz = sc->nz - 1;
    return sc->den[(size_t)ix + (size_t)sc->nx * ((size_t)iy + (size_t)sc->ny * iz)];
}

/* ---------------------------------------------------------------- source */
/* getPositionFromShape, gPET_kernals.cu:445-482 */
static void shape_position(const or_scene* sc, int si, stream_t* st, real p[3])
{
    const float* c = sc->src_coef + 6 * si;
    int shape = sc->src_shape[si];
    if (shape < 0 || shape > 2) shape = 0;
    if (shape == 0) {
        real a = st_u(st), b = st_u(st), d = st_u(st);
        p[0] = (real)c[0] + (real)c[3] * ((real)-1.0 + (real)2.0 * a) * (real)0.5;
        p[1] = (real)c[1] + (real)c[4] * ((real)-1.0 + (real)2.0 * b) * (real)0.5;
        p[2] = (real)c[2] + (real)c[5] * ((real)-1.0 + (real)2.0 * d) * (real)0.5;
    } else if (shape == 1) {
        real phi = st_u(st);
        real r = (real)c[3] * R_SQRT(st_u(st));
        real zz = st_u(st);
        real s, cs;
        r_sincos_turns(phi, &s, &cs);
        p[0] = (real)c[0] + r * cs;
        p[1] = (real)c[1] + r * s;
        p[2] = (real)c[2] + (real)c[4] * ((real)-1.0 + (real)2.0 * zz) * (real)0.5;
    } else {
        real phi = st_u(st);
        real cost = (real)-1.0 + (real)2.0 * st_u(st);
        real r = (real)c[3] * R_CBRT(st_u(st));
        real s, cs;
        r_sincos_turns(phi, &s, &cs);
        real st2 = R_SQRT((real)1.0 - cost * cost);
        p[0] = (real)c[0] + r * st2 * cs;
        p[1] = (real)c[1] + r * st2 * s;
        p[2] = (real)c[2] + r * cost;
    }
}

/* sampleEkPositron, gPET_kernals.cu:420-443: rejection on the fitted
 * spectrum polynomial (evaluated by Horner); returns kinetic energy in eV */
static real sample_ek(const or_scene* sc, int type, stream_t* st)
{
    const float* cf = sc->iso_coef + 8 * type;
    real e = (real)0.0;
    for (int it = 0; it < 100000; ++it) {
        e = st_u(st) * ((real)cf[0] - (real)0.511) + (real)0.511;
        real u = (real)cf[1] * st_u(st);
        real sum = (real)cf[2];
        for (int k = 3; k < 8; ++k) sum = sum * e + (real)cf[k];
        if (!(u > sum)) break;
    }
    return (e - (real)0.511) * (real)1.0e6;
}

/* The positron-range walk below ends where the density-weighted path length
 * reaches r. Where every voxel it reads has one density rho, that end point
 * is x + (r / rho) * d / r exactly; the walk reads voxels within
 * floor(L / dmin) + 2 (Chebyshev) of its start voxel, L = r / rho (the end
 * voxel and the one entered beyond it). The map holds, per voxel, the largest
 * R <= OR_PRMAX such that all voxels within R have its density (same float
 * bits) and lie in [1, n-2] on every axis (-1 where the voxel itself does
 * not), so with L < (R - 1.5) * dmin the closed form replaces the walk. The
 * CUDA kernels take the same closed form under the same test, so both give
 * the same end point bit for bit; against the reference's walk it differs by
 * rounding only. */
#define OR_PRMAX 6

static inline int pr_interior(int x, int y, int z, int nx, int ny, int nz)
{
    return x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 && z >= 1 && z <= nz - 2;
}

/* the map of the scene's phantom into out[nx*ny*nz]: Jacobi passes of
 * m(v) = 1 + min over the 26 neighbours, valid where v and its neighbours
 * are in range and of one density (the ball of radius R around v is the union
 * of the balls of radius R-1 around its neighbours) */
void oracle_build_prmap(const or_scene* sc, int8_t* out)
{
    const int nx = sc->nx, ny = sc->ny, nz = sc->nz;
    const int64_t n = (int64_t)nx * ny * nz;
    int8_t* tmp = (int8_t*)malloc((size_t)n);
    int8_t* m[2] = {out, tmp};
    int cur = (OR_PRMAX - 1) % 2;
    #pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < n; ++v) {
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((int64_t)nx * ny));
        int8_t r = -1;
        if (pr_interior(x, y, z, nx, ny, nz)) {
            uint32_t b;
            memcpy(&b, sc->den + v, 4);
            r = 1;
            for (int dz = -1; dz <= 1 && r; ++dz)
                for (int dy = -1; dy <= 1 && r; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        uint32_t q;
                        memcpy(&q, sc->den + v + dx + (int64_t)nx * (dy + (int64_t)ny * dz), 4);
                        if (!pr_interior(x + dx, y + dy, z + dz, nx, ny, nz) || q != b) { r = 0; break; }
                    }
        }
        m[cur][v] = r;
    }
    for (int pass = 1; pass < OR_PRMAX; ++pass) {
        const int8_t* m0 = m[cur];
        int8_t* m1 = m[cur ^ 1];
        #pragma omp parallel for schedule(static)
        for (int64_t v = 0; v < n; ++v) {
            int r = m0[v];
            if (r >= 1) {
                const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((int64_t)nx * ny));
                int mn = OR_PRMAX;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            if ((dx | dy | dz) == 0) continue;
                            int q = m0[(int64_t)(x + dx) + (int64_t)nx * ((y + dy) + (int64_t)ny * (z + dz))];
                            if (q < mn) mn = q;
                        }
                r = mn + 1 < OR_PRMAX ? mn + 1 : OR_PRMAX;
            }
            m1[v] = (int8_t)r;
        }
        cur ^= 1;
    }
    free(tmp);
}

/* the closed form above; returns 0 where the walk is needed. A walk that
 * reaches beyond the uniform cube (R >= 2) starts where its first
 * lim = (R - 1.5) * dmin of path takes it: x moves by lim along d / r and *s0 =
 * lim * rho is the density-weighted length already covered (up to there the
 * walk reads only voxels of density rho: the voxel holding that point lies
 * within R - 1 of the start voxel, the one entered after it within R);
 * otherwise x is unchanged and *s0 = 0. A zero displacement moves nothing, as
 * in the walk. */
static int prange_uniform(const or_scene* sc, real x[3], const real d[3], real r, real* s0)
{
    *s0 = (real)0.0;
    if (!(r > (real)0.0)) return 1;
    if (!sc->prmap) return 0;
    int ix, iy, iz;
    if (!abs_vox(sc, (real)(1.0f / sc->dx), (real)(1.0f / sc->dy), (real)(1.0f / sc->dz), x[0], x[1], x[2],
                 &ix, &iy, &iz))
        return 0;
    const size_t i = (size_t)ix + (size_t)sc->nx * ((size_t)iy + (size_t)sc->ny * iz);
    const int R = sc->prmap[i];
    const real rho = (real)sc->den[i];
    if (!(rho > (real)0.0) || R < 2) return 0;
    const real L = r / rho;
    const real dmin = (real)fminf(sc->dx, fminf(sc->dy, sc->dz));
    const real lim = ((real)R - (real)1.5) * dmin;
    const real ir = (real)1.0 / r;
    const real dn0 = d[0] * ir, dn1 = d[1] * ir, dn2 = d[2] * ir;
    if (L < lim) {
        x[0] = x[0] + L * dn0;
        x[1] = x[1] + L * dn1;
        x[2] = x[2] + L * dn2;
        return 1;
    }
    x[0] = x[0] + lim * dn0;
    x[1] = x[1] + lim * dn1;
    x[2] = x[2] + lim * dn2;
    *s0 = lim * rho;
    return 0;
}

/* setPositronRange, gPET_kernals.cu:347-418: Gaussian displacement with
 * sigma = Rex/2 (Rex from a water fit), walked through voxels so that the
 * density-weighted length equals r. The density is read from the voxel being
 * entered (as the reference does). A positron that reaches outside the phantom
 * finishes its remaining range in air (0.0012905 g/cm^3); the reference adds a
 * spurious 1000 cm there (:383,405). */
/* spare (may be NULL): the second normal of the last Box-Muller pair, which
 * the pair emission uses for its non-collinearity angle */
static void positron_range(const or_scene* sc, real x[3], real ek, const real* dir, stream_t* st, real* spare)
{
    real ekin = ek / (real)1.0e6;
    real b1 = (real)5.44040782, b2 = (real)0.369516529;
    real rex = (real)0.1 * b1 * ekin * ekin / (b2 + ekin);
    real sigma = rex / (real)2.0;
    real d[3];
    {
        real n1, n2;
        st_normal2(st, &n1, &n2);
        d[0] = sigma * n1;
        d[1] = sigma * n2;
        real n3, n4;
        st_normal2(st, &n3, &n4);
        d[2] = sigma * n3;
        if (spare) *spare = n4;
    }
    real r = R_SQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (dir) {
        real tmp = R_SQRT(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        d[0] = r * dir[0] / tmp; d[1] = r * dir[1] / tmp; d[2] = r * dir[2] / tmp;
    }
    real s0;
    if (prange_uniform(sc, x, d, r, &s0)) return;
    /* the walk multiplies by reciprocals computed once */
    const real id0 = (real)1.0 / d[0], id1 = (real)1.0 / d[1], id2 = (real)1.0 / d[2];
    const real ir = (real)1.0 / r;
    const real dn0 = d[0] * ir, dn1 = d[1] * ir, dn2 = d[2] * ir;
    real idx = (real)1.0 / (real)sc->dx, idy = (real)1.0 / (real)sc->dy, idz = (real)1.0 / (real)sc->dz;
    int vx = 0, vy = 0, vz = 0;
    int inside = abs_vox(sc, (real)(1.0f / sc->dx), (real)(1.0f / sc->dy), (real)(1.0f / sc->dz),
                         x[0], x[1], x[2], &vx, &vy, &vz);
    (void)idx; (void)idy; (void)idz;
    if (!inside) {
        /* the reference keeps the truncated indices even when outside; they
         * are only used while inside, so any value will do */
        vx = vy = vz = 0;
    }
    real s = s0, step;
    const real xmax = (real)sc->offx + (real)sc->nx * (real)sc->dx;
    const real ymax = (real)sc->offy + (real)sc->ny * (real)sc->dy;
    const real zmax = (real)sc->offz + (real)sc->nz * (real)sc->dz;
    for (int guard = 0; s < r && guard < 100000; ++guard) {
        step = (real)1000.0;
        if (inside) {
            int ax = 0;
            real bb = ((real)sc->offx + (real)(vx + (d[0] > (real)0.0)) * (real)sc->dx - x[0]) * id0;
            if (step > bb) { step = bb; ax = 1; }
            bb = ((real)sc->offy + (real)(vy + (d[1] > (real)0.0)) * (real)sc->dy - x[1]) * id1;
            if (step > bb) { step = bb; ax = 2; }
            bb = ((real)sc->offz + (real)(vz + (d[2] > (real)0.0)) * (real)sc->dz - x[2]) * id2;
            if (step > bb) { step = bb; ax = 3; }
            if (ax == 1) vx += d[0] > (real)0.0 ? 1 : -1;
            else if (ax == 2) vy += d[1] > (real)0.0 ? 1 : -1;
            else vz += d[2] > (real)0.0 ? 1 : -1;
            real rho = (real)den_clamped(sc, vx, vy, vz);
            step = step * r;
            s += step * rho;
            if (s > r) step += (r - s) / rho;
        } else {
            step = (r - s) / (real)0.0012905;
            s = r + (real)100.0;
        }
        x[0] += step * dn0;
        x[1] += step * dn1;
        x[2] += step * dn2;
        if (x[0] < (real)sc->offx || x[0] > xmax) inside = 0;
        if (x[1] < (real)sc->offy || x[1] > ymax) inside = 0;
        if (x[2] < (real)sc->offz || x[2] > zmax) inside = 0;
    }
}

/* ------------------------------------------------------ phantom transport */
typedef struct {
    real x[3], u[3], E;
    double t;
    real tf;
    int nscat;
} photon_t;

/* comsam(matid), gPET_kernals.cu:66-88: cos(theta) from the Compton surface */
static inline void compton_surface(const or_scene* sc, real e, int m, stream_t* st, real* efrac, real* cost)
{
    real indcp = st_u(st) * (real)sc->idcp_c;
    real inde = e * (real)sc->ide_c;
    real c = lerp2(sc->cmpsf + (size_t)m * sc->ncp_c * sc->ne_c, sc->ncp_c, sc->ne_c, inde, indcp);
    if (c > (real)1.0) c = (real)1.0;
    if (c < (real)-1.0) c = (real)-1.0;
    *cost = c;
    *efrac = (real)1.0 / ((real)1.0 + e * C_IMC2 * ((real)1.0 - c));
}

/* rylsam, gPET_kernals.cu:128-146 */
static inline real rayleigh_surface(const or_scene* sc, real e, int m, stream_t* st)
{
    real indcp = st_u(st) * (real)sc->idcp_r;
    real inde = e * (real)sc->ide_r;
    real c = lerp2(sc->rayff + (size_t)m * sc->ncp_r * sc->ne_r, sc->ncp_r, sc->ne_r, inde, indcp);
    if (c > (real)1.0) c = (real)1.0;
    if (c < (real)-1.0) c = (real)-1.0;
    return c;
}

/* photon(), gPET_kernals.cu:256-345. Returns status: 0 photoelectric,
 * 1 escaped the phantom (or dropped below eabsph after a Compton event and
 * leaves as-is, :318-320), 3 step cap */
static int phantom_transport(const or_scene* sc, const wck_t* wck, photon_t* p, stream_t* st)
{
    const real idx = (real)(1.0f / sc->dx), idy = (real)(1.0f / sc->dy), idz = (real)(1.0f / sc->dz);
    for (int step = 0; step < MAX_STEPS; ++step) {
        real lammin = wck_at(wck, p->E);
        real s = -lammin * R_LOG(st_u(st));
        p->x[0] = R_FMA(s, p->u[0], p->x[0]);
        p->x[1] = R_FMA(s, p->u[1], p->x[1]);
        p->x[2] = R_FMA(s, p->u[2], p->x[2]);
        TIME_STEP(p, s);
        int ix, iy, iz;
        if (!abs_vox(sc, idx, idy, idz, p->x[0], p->x[1], p->x[2], &ix, &iy, &iz)) return 1;
        size_t v = (size_t)ix + (size_t)sc->nx * ((size_t)iy + (size_t)sc->ny * iz);
        real voxden = (real)sc->den[v];
        int m = sc->mat[v];
        real lamden = lammin * voxden;
        real prob = R_FMA(-lamden, xs_at(sc, sc->lamph, m, p->E), (real)1.0);
        real rn = st_u(st);
        if (rn < prob) continue;
        prob = R_FMA(lamden, xs_at(sc, sc->compt, m, p->E), prob);
        if (rn < prob) {
            real efrac, cost;
            compton_surface(sc, p->E, m, st, &efrac, &cost);
            real phi = st_u(st);
            p->E *= efrac;
            p->nscat++;
            if (p->E < (real)sc->eabsph) return 1;
            rotate(&p->u[0], &p->u[1], &p->u[2], cost, phi);
            continue;
        }
        prob = R_FMA(lamden, xs_at(sc, sc->rayle, m, p->E), prob);
        if (rn < prob) {
            real cost = rayleigh_surface(sc, p->E, m, st);
            real phi = st_u(st);
            rotate(&p->u[0], &p->u[1], &p->u[2], cost, phi);
            p->nscat++;
            continue;
        }
        return 0;
    }
    return 3;
}

/* ------------------------------------------------------ detector transport */
typedef struct {
    real x[3], u[3], E;
    double t;
    real tf;
    int panel;          /* index into the panel array */
} local_t;

/* panel search of photonde, gPET_kernals.cu:963-1009: first panel (in order)
 * whose plane the photon crosses within the panel face while moving along the
 * panel's depth direction; the photon is moved onto that plane */
static int enter_panel(const or_scene* sc, const photon_t* p, local_t* q)
{
    for (int i = 0; i < sc->npanels; ++i) {
        const float* P = sc->panels + (size_t)i * OR_PANEL_STRIDE;
        real px = p->x[0] - (real)P[15], py = p->x[1] - (real)P[16], pz = p->x[2] - (real)P[17];
        real tx = px * (real)P[21] + py * (real)P[22] + pz * (real)P[23];
        real ty = px * (real)P[24] + py * (real)P[25] + pz * (real)P[26];
        real tz = px * (real)P[27] + py * (real)P[28] + pz * (real)P[29];
        real tvx = p->u[0] * (real)P[21] + p->u[1] * (real)P[22] + p->u[2] * (real)P[23];
        real tvy = p->u[0] * (real)P[24] + p->u[1] * (real)P[25] + p->u[2] * (real)P[26];
        real tvz = p->u[0] * (real)P[27] + p->u[1] * (real)P[28] + p->u[2] * (real)P[29];
        if (tvx * (real)P[18] >= (real)0.0) {
            real ty2 = ty - tx / tvx * tvy;
            real tz2 = tz - tx / tvx * tvz;
            if (R_FABS(ty2) < (real)P[1] / (real)2.0 && R_FABS(tz2) < (real)P[2] / (real)2.0) {
                q->x[0] = (real)0.0; q->x[1] = ty2; q->x[2] = tz2;
                q->u[0] = tvx; q->u[1] = tvy; q->u[2] = tvz;
                q->E = p->E;
#ifdef ORACLE_FP32
                q->t = p->t + (double)(p->tf + -tx / tvx * DM_INV_SPEED);
#else
                q->t = p->t + (double)(-tx) / (C_SPE * (double)tvx);
#endif
                q->tf = (real)0.0;
                q->panel = i;
                return 1;
            }
        }
    }
    return 0;
}

/* crystalSearch, gPET_kernals.cu:1236-1279: m_id 0 crystal, 1 gap; inside
 * quadratic surface k: gap (the reference), or crystal of the extra material
 * 2 + k when the detector lists one */
static void crystal_search(const or_scene* sc, const float* P, const real x[3], int* m_id, int* M_id, int* L_id)
{
    real xx = x[0], y = x[1], z = x[2];
    int region = 0;
    for (int k = 0; k < sc->nsurface; ++k) {
        const float* a = sc->surface + 10 * k;
        real v = (real)a[0] * xx * xx + (real)a[1] * y * y + (real)a[2] * z * z + (real)a[3] * xx * y +
                 (real)a[4] * xx * z + (real)a[5] * y * z + (real)a[6] * xx + (real)a[7] * y + (real)a[8] * z +
                 (real)a[9];
        if (v < (real)0.0) {
            if (k < sc->nxdet) { region = 2 + k; break; }
            *m_id = 1;
            return;
        }
    }
    y = (real)P[1] / (real)2.0 + x[1];
    z = (real)P[2] / (real)2.0 + x[2];
    real pmy = (real)P[4] + (real)P[7], pmz = (real)P[5] + (real)P[8];
    int my = R_FLOOR(y / pmy) > (real)0.0 ? (int)(y / pmy) : 0;
    int mz = R_FLOOR(z / pmz) > (real)0.0 ? (int)(z / pmz) : 0;
    *M_id = mz * sc->moduleNy + my;
    y = y - (real)my * pmy;
    z = z - (real)mz * pmz;
    if (y > (real)P[4] || z > (real)P[5]) { *m_id = 1; return; }
    real pcy = (real)P[10] + (real)P[13], pcz = (real)P[11] + (real)P[14];
    int ly = R_FLOOR(y / pcy) > (real)0.0 ? (int)(y / pcy) : 0;
    int lz = R_FLOOR(z / pcz) > (real)0.0 ? (int)(z / pcz) : 0;
    *L_id = lz * sc->crystalNy + ly;
    y = y - (real)ly * pcy;
    z = z - (real)lz * pcz;
    if (y > (real)P[10] || z > (real)P[11]) { *m_id = 1; return; }
    *m_id = region;
}

/* comsam (free electron Klein-Nishina), gPET_kernals.cu:90-126 */
static void kn_sample(real e, stream_t* st, real* efrac, real* cost)
{
    real e0 = e * C_IMC2;
    real twoe = (real)2.0 * e0;
    real kmin2 = (real)1.0 / (((real)1.0 + twoe) * ((real)1.0 + twoe));
    real loge = R_LOG((real)1.0 + twoe);
    real ef = (real)1.0;
    for (int it = 0; it < 100000; ++it) {
        if (st_u(st) * (loge + twoe * ((real)1.0 + e0) * kmin2) < loge)
            ef = R_EXP(-st_u(st) * loge);
        else
            ef = R_SQRT(kmin2 + st_u(st) * ((real)1.0 - kmin2));
        real mess = e0 * e0 * ef * ((real)1.0 + ef * ef);
        if (st_u(st) * mess <= mess - ((real)1.0 - ef) * (((real)1.0 + twoe) * ef - (real)1.0)) break;
    }
    *efrac = ef;
    *cost = (real)1.0 - ((real)1.0 - ef) / (ef * e0);
}

/* adder, gPET_kernals.cu:737-755: same crystal -> energy-weighted centroid
 * and summed energy, first time kept */
static int adder(or_event* ev, int* n, const or_event* e)
{
    for (int i = 0; i < *n; ++i) {
        if (e->siten == ev[i].siten) {
            float s = ev[i].E + e->E;
            ev[i].x = (ev[i].x * ev[i].E + e->x * e->E) / s;
            ev[i].y = (ev[i].y * ev[i].E + e->y * e->E) / s;
            ev[i].z = (ev[i].z * ev[i].E + e->z * e->E) / s;
            ev[i].E = ev[i].E + e->E;
            return 1;
        }
    }
    if (*n >= MAX_PULSE) return 0;
    ev[(*n)++] = *e;
    return 1;
}

/* readout, gPET_kernals.cu:756-813. Depth 3 leaves the pulses as they are
 * (the reference returns early there and then copies a stale count of 4). */
static int readout(const or_scene* sc, or_event* ev, int n, or_event* out)
{
    int depth = sc->rdepth, policy = sc->rpolicy;
    if (depth == 3) {
        for (int i = 0; i < n; ++i) out[i] = ev[i];
        return n;
    }
    if (policy == 1) depth = 2;
    for (int i = 0; i < n; ++i) {
        if (depth == 0) ev[i].siten = 0;
        else if (depth == 1) ev[i].siten = ev[i].pann;
        else if (depth == 2) ev[i].siten = ev[i].pann * sc->moduleN + ev[i].modn;
    }
    uint8_t dead[MAX_PULSE];
    memset(dead, 0, sizeof(dead));
    int k = 0;
    for (int i = 0; i < n; ++i) {
        if (dead[i]) continue;
        or_event e0 = ev[i];
        for (int j = i + 1; j < n; ++j) {
            const or_event* e = &ev[j];
            if (e->parn == e0.parn && e->siten == e0.siten) {
                if (policy == 1) {
                    float s = e0.E + e->E;
                    e0.x = (e0.x * e0.E + e->x * e->E) / s;
                    e0.y = (e0.y * e0.E + e->y * e->E) / s;
                    e0.z = (e0.z * e0.E + e->z * e->E) / s;
                    e0.E = e0.E + e->E;
                } else {
                    e0 = (e0.E > e->E) ? e0 : *e;
                }
                dead[j] = 1;
            }
        }
        out[k++] = e0;
    }
    return k;
}

typedef struct {
    or_event* ev; uint8_t* scat; uint8_t* slot; int64_t n, cap;
    int32_t* hid; float* hf; int64_t nh, caph;
    int64_t n_entered, n_pairs, n_overflow, n_stepcap;
} tbuf_t;

static void tb_push_pulse(tbuf_t* b, const or_event* e, uint8_t scat, uint8_t slot)
{
    if (b->n == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 1024;
        b->ev = (or_event*)realloc(b->ev, sizeof(or_event) * b->cap);
        b->scat = (uint8_t*)realloc(b->scat, b->cap);
        b->slot = (uint8_t*)realloc(b->slot, b->cap);
    }
    b->ev[b->n] = *e; b->scat[b->n] = scat; b->slot[b->n] = slot; b->n++;
}

static void tb_push_hit(tbuf_t* b, const int32_t id[5], const float f[5])
{
    if (b->nh == b->caph) {
        b->caph = b->caph ? 2 * b->caph : 1024;
        b->hid = (int32_t*)realloc(b->hid, sizeof(int32_t) * 5 * b->caph);
        b->hf = (float*)realloc(b->hf, sizeof(float) * 5 * b->caph);
    }
    memcpy(b->hid + 5 * b->nh, id, 20);
    memcpy(b->hf + 5 * b->nh, f, 20);
    b->nh++;
}

/* photonde per photon, gPET_kernals.cu:1011-1200 */
static void detector_transport(const or_scene* sc, const wck_t* wck, local_t* q, int32_t parn, int32_t eventid,
                               int scat, stream_t* st, tbuf_t* tb, int rec_hits)
{
    const float* P = sc->panels + (size_t)q->panel * OR_PANEL_STRIDE;
    const int32_t pann = (int32_t)P[30];
    or_event ev[MAX_PULSE];
    int nev = 0, overflow = 0, nh = 0;
    int step;
    for (step = 0; step < MAX_STEPS; ++step) {
        real lammin = wck_at(wck, q->E);
        real s = -lammin * R_LOG(st_u(st));
        q->x[0] = R_FMA(s, q->u[0], q->x[0]);
        q->x[1] = R_FMA(s, q->u[1], q->x[1]);
        q->x[2] = R_FMA(s, q->u[2], q->x[2]);
        TIME_STEP(q, s);
        if (R_FABS(q->x[1]) > (real)P[1] * (real)0.5 || R_FABS(q->x[2]) > (real)P[2] * (real)0.5 ||
            q->x[0] * (real)P[18] < (real)0.0 || q->x[0] * (real)P[18] > (real)P[0])
            break;
        int m_id = -1, M_id = -1, L_id = -1;
        crystal_search(sc, P, q->x, &m_id, &M_id, &L_id);
        real den = (real)(m_id < 2 ? sc->det_den[m_id] : sc->xdet_den[m_id - 2]);
        int mat = m_id < 2 ? sc->det_mat[m_id] : sc->xdet_mat[m_id - 2];
        real lamden = lammin * den;
        real prob = R_FMA(-lamden, xs_at(sc, sc->lamph, mat, q->E), (real)1.0);
        if (prob < (real)0.0) prob = (real)0.0;
        real rn = st_u(st);
        if (rn < prob) continue;
        prob = R_FMA(lamden, xs_at(sc, sc->compt, mat, q->E), prob);
        int type = 0;
        real dep = (real)0.0;
        int stop = 0;
        if (rn < prob) {
            real efrac, cost;
            kn_sample(q->E, st, &efrac, &cost);
            real de = q->E * ((real)1.0 - efrac);
            real phi = st_u(st);
            if (m_id != 1) {   /* a crystal (not the gap) */
                or_event e;
                e.parn = parn; e.cryn = L_id; e.modn = M_id; e.pann = pann;
                e.siten = pann * sc->moduleN * sc->crystalN + M_id * sc->crystalN + L_id;
                e.eventid = eventid;
                e.E = (float)de; e.t = q->t + (double)q->tf;
                e.x = (float)q->x[0]; e.y = (float)q->x[1]; e.z = (float)q->x[2];
                if (rec_hits) {
                    int32_t hid[5] = {parn, pann, M_id, L_id, 1};
                    float hf[5] = {(float)de, (float)e.t, (float)q->x[0], (float)q->x[1], (float)q->x[2]};
                    if (nh < MAX_HITS) { tb_push_hit(tb, hid, hf); nh++; } else overflow = 1;
                }
                if (!adder(ev, &nev, &e)) overflow = 1;
            }
            q->E -= de;
            if (q->E < (real)sc->eabsph) {
                type = 2; dep = q->E; stop = 1;
            } else {
                rotate(&q->u[0], &q->u[1], &q->u[2], cost, phi);
                continue;
            }
        } else {
            prob = R_FMA(lamden, xs_at(sc, sc->rayle, mat, q->E), prob);
            if (rn < prob) {
                real cost = rayleigh_surface(sc, q->E, mat, st);
                real phi = st_u(st);
                rotate(&q->u[0], &q->u[1], &q->u[2], cost, phi);
                continue;
            }
            type = 4; dep = q->E; stop = 1;
        }
        if (stop) {
            if (m_id != 1) {   /* a crystal (not the gap) */
                or_event e;
                e.parn = parn; e.cryn = L_id; e.modn = M_id; e.pann = pann;
                e.siten = pann * sc->moduleN * sc->crystalN + M_id * sc->crystalN + L_id;
                e.eventid = eventid;
                e.E = (float)dep; e.t = q->t + (double)q->tf;
                e.x = (float)q->x[0]; e.y = (float)q->x[1]; e.z = (float)q->x[2];
                if (rec_hits) {
                    int32_t hid[5] = {parn, pann, M_id, L_id, type};
                    float hf[5] = {(float)dep, (float)e.t, (float)q->x[0], (float)q->x[1], (float)q->x[2]};
                    if (nh < MAX_HITS) { tb_push_hit(tb, hid, hf); nh++; } else overflow = 1;
                }
                if (!adder(ev, &nev, &e)) overflow = 1;
            }
            break;
        }
    }
    if (step == MAX_STEPS) tb->n_stepcap++;
    if (overflow) tb->n_overflow++;
    if (nev) {
        or_event out[MAX_PULSE];
        int k = readout(sc, ev, nev, out);
        for (int i = 0; i < k; ++i) tb_push_pulse(tb, &out[i], (uint8_t)(scat != 0), (uint8_t)i);
    }
}

/* --------------------------------------------------------- one decay */
typedef struct {
    wck_t wph, wdet;
    double ntau_us[64], cfac[64];   /* per source: -lifetime (us), 1 - exp(-dt/lifetime) */
} prep_t;

/* spare: a standard normal already drawn (the positron range's second
 * normal of its last pair) for the non-collinearity angle, or NULL */
static void make_pair(const or_scene* sc, stream_t* st, const real pos[3], photon_t ph[2], double t_us,
                      const real* spare)
{
    /* setPosition, gPET_kernals.cu:536-555 */
    real cost = (real)-1.0 + (real)2.0 * st_u(st);
    real phi = st_u(st);
    real s, c;
    r_sincos_turns(phi, &s, &c);
    real sint = R_SQRT((real)1.0 - cost * cost);
    real u0 = sint * c, u1 = sint * s, u2 = cost;
    real phi2 = st_u(st);
    real theta = (spare ? *spare : st_normal(st)) * (real)sc->noncol_sigma;
    for (int k = 0; k < 2; ++k) {
        ph[k].x[0] = pos[0]; ph[k].x[1] = pos[1]; ph[k].x[2] = pos[2];
        ph[k].t = t_us; ph[k].tf = (real)0.0; ph[k].nscat = 0;
    }
    ph[0].u[0] = u0; ph[0].u[1] = u1; ph[0].u[2] = u2;
    ph[0].E = C_MC2 + theta * C_MC2 / (real)2.0;
    real ts, tc;
    r_sincos_turns(theta * (real)0.159154943091895335768883763, &ts, &tc);  /* cos(theta) */
    (void)ts;
    rotate(&u0, &u1, &u2, -tc, phi2);
    ph[1].u[0] = u0; ph[1].u[1] = u1; ph[1].u[2] = u2;
    ph[1].E = C_MC2 - theta * C_MC2 / (real)2.0;
}

static void record_exit(or_exit* ex, const photon_t* p, int status, int panel)
{
    ex->x = (float)p->x[0]; ex->y = (float)p->x[1]; ex->z = (float)p->x[2];
    ex->ux = (float)p->u[0]; ex->uy = (float)p->u[1]; ex->uz = (float)p->u[2];
    ex->E = (float)p->E; ex->t = p->t + (double)p->tf; ex->nscat = p->nscat; ex->status = status; ex->panel = panel;
}

static void record_src(or_src* s, const photon_t* p, int64_t d)
{
    s->x = (float)p->x[0]; s->y = (float)p->x[1]; s->z = (float)p->x[2];
    s->ux = (float)p->u[0]; s->uy = (float)p->u[1]; s->uz = (float)p->u[2];
    s->E = (float)p->E; s->eventid = (int32_t)d; s->t = p->t;
}

static void transport_pair(const or_scene* sc, const prep_t* pp, int64_t d, photon_t ph[2], int have,
                           or_exit* exits, or_src* src, tbuf_t* tb, int flags)
{
    for (int k = 0; k < 2; ++k) {
        if (src) {
            if (have) record_src(&src[k], &ph[k], d);
            else memset(&src[k], 0, sizeof(or_src));
        }
        if (!have) {
            if (exits) { photon_t z; memset(&z, 0, sizeof(z)); record_exit(&exits[k], &z, 2, -1); }
            continue;
        }
        stream_t st;
        st_init(&st, sc, TAG_PHANTOM + k, (uint64_t)d);
        int status = phantom_transport(sc, &pp->wph, &ph[k], &st);
        int panel = -1;
        local_t q;
        if (status == 3) tb->n_stepcap++;
        if (status == 1 && enter_panel(sc, &ph[k], &q)) {
            panel = q.panel;
            tb->n_entered++;
            stream_t sd;
            st_init(&sd, sc, TAG_DET + k, (uint64_t)d);
            detector_transport(sc, &pp->wdet, &q, (int32_t)(2 * d + k), (int32_t)d, ph[k].nscat, &sd, tb,
                               flags & 2);
        }
        if (exits) record_exit(&exits[k], &ph[k], status, panel);
    }
}

static void simulate_decay(const or_scene* sc, const prep_t* pp, int64_t d, or_exit* exits, or_src* src, tbuf_t* tb,
                           int flags)
{
    stream_t st;
    st_init(&st, sc, TAG_DECAY, (uint64_t)d);
    photon_t ph[2];
    int have = 0;
    if (sc->npsf > 0) {
        /* setPositionForPhoton / photon PSF, gPET.cu:13-199, gPET_kernals.cu:563-604 */
        const double* r = sc->psf + 8 * d;
        if (sc->psf_ptype == 1) {
            ph[0].x[0] = (real)(float)r[0]; ph[0].x[1] = (real)(float)r[1]; ph[0].x[2] = (real)(float)r[2];
            ph[0].u[0] = (real)(float)r[4]; ph[0].u[1] = (real)(float)r[5]; ph[0].u[2] = (real)(float)r[6];
            ph[0].E = (real)(float)r[7]; ph[0].t = r[3]; ph[0].tf = (real)0.0; ph[0].nscat = 0;
            /* one photon per record: photon slot 1 carries nothing */
            if (src) {
                if (r[3] > 0.0 && ph[0].E >= (real)0.0) record_src(&src[0], &ph[0], d);
                else memset(&src[0], 0, sizeof(or_src));
                memset(&src[1], 0, sizeof(or_src));
            }
            stream_t s0;
            st_init(&s0, sc, TAG_PHANTOM, (uint64_t)d);
            int status = r[3] > 0.0 && ph[0].E >= (real)0.0 ? phantom_transport(sc, &pp->wph, &ph[0], &s0) : 2;
            int panel = -1;
            local_t q;
            if (status == 3) tb->n_stepcap++;
            if (status == 1 && enter_panel(sc, &ph[0], &q)) {
                panel = q.panel;
                tb->n_entered++;
                stream_t sd;
                st_init(&sd, sc, TAG_DET, (uint64_t)d);
                detector_transport(sc, &pp->wdet, &q, (int32_t)(2 * d), (int32_t)d, ph[0].nscat, &sd, tb, flags & 2);
            }
            if (exits) {
                if (status == 2) { photon_t z; memset(&z, 0, sizeof(z)); record_exit(&exits[0], &z, 2, -1); }
                else record_exit(&exits[0], &ph[0], status, panel);
                photon_t z; memset(&z, 0, sizeof(z)); record_exit(&exits[1], &z, 2, -1);
            }
            return;
        }
        real pos[3] = {(real)(float)r[0], (real)(float)r[1], (real)(float)r[2]};
        real dir[3] = {(real)(float)r[4], (real)(float)r[5], (real)(float)r[6]};
        real spare = (real)0.0;
        if (sc->useprange) positron_range(sc, pos, (real)(float)r[7], dir, &st, &spare);
        make_pair(sc, &st, pos, ph, r[3], sc->useprange ? &spare : NULL);
        have = 1;
        tb->n_pairs++;
        transport_pair(sc, pp, d, ph, have, exits, src, tb, flags);
        return;
    }
    /* source mode: decay d belongs to the source whose index range holds it */
    int si = 0;
    while (si < sc->nsrc - 1 && d >= sc->src_first[si] + sc->src_count[si]) si++;
    int type = sc->src_type[si];
    /* truncated exponential decay time in [0, dt) (the per-atom test of
     * setPosition, gPET_kernals.cu:519-521, conditioned on decaying) */
    double ud = st_ud(&st);
    const double xl = -ud * pp->cfac[si];
    /* t = tstart - lifetime log(1 - u (1 - exp(-window / lifetime))), in us */
#ifdef ORACLE_FP32
    const double L = pp->cfac[si] <= 0.015625 ? dm_log1p_small(xl) : dm_log(1.0 + xl);
#else
    const double L = log1p(xl);
#endif
    double t_us = dm_fmad(pp->ntau_us[si], L, sc->tstart_s * 1e6);
    real br = st_u(&st);
    if (br < (real)sc->iso_ratio[type]) {
        real pos[3];
        shape_position(sc, si, &st, pos);
        real spare = (real)0.0;
        if (sc->useprange) {
            real ek = sample_ek(sc, type, &st);
            positron_range(sc, pos, ek, NULL, &st, &spare);
        }
        make_pair(sc, &st, pos, ph, t_us, sc->useprange ? &spare : NULL);
        have = 1;
        tb->n_pairs++;
    }
    transport_pair(sc, pp, d, ph, have, exits, src, tb, flags);
}

/* ------------------------------------------------------------- digitizer */
typedef struct { or_event e; uint8_t scat, slot; int32_t site; } dpulse_t;

/* total order used for the per-site dead-time pass: (site, t, parn, slot) */
static int cmp_site_t(const void* a, const void* b)
{
    const dpulse_t* x = (const dpulse_t*)a;
    const dpulse_t* y = (const dpulse_t*)b;
    if (x->site != y->site) return x->site < y->site ? -1 : 1;
    if (x->e.t != y->e.t) return x->e.t < y->e.t ? -1 : 1;
    if (x->e.parn != y->e.parn) return x->e.parn < y->e.parn ? -1 : 1;
    return (int)x->slot - (int)y->slot;
}

/* total order of the singles list: (t, parn, slot) */
static int cmp_t(const void* a, const void* b)
{
    const dpulse_t* x = (const dpulse_t*)a;
    const dpulse_t* y = (const dpulse_t*)b;
    if (x->e.t != y->e.t) return x->e.t < y->e.t ? -1 : 1;
    if (x->e.parn != y->e.parn) return x->e.parn < y->e.parn ? -1 : 1;
    return (int)x->slot - (int)y->slot;
}

static int cmp_parn_slot(const void* a, const void* b)
{
    const dpulse_t* x = (const dpulse_t*)a;
    const dpulse_t* y = (const dpulse_t*)b;
    if (x->e.parn != y->e.parn) return x->e.parn < y->e.parn ? -1 : 1;
    return (int)x->slot - (int)y->slot;
}

/* blur, gPET_kernals.cu:814-837, with the normal deviates drawn from the
 * pulse's own Philox stream (key (parn, slot)) so the result does not depend
 * on the order pulses are processed in */
static void blur_event(const or_scene* sc, or_event* e, stream_t* st)
{
    float R = 0.0f;
    if (sc->blurpolicy == 0) R = dm_sqrt(sc->Eref / e->E) * sc->Rref;
    if (sc->blurpolicy == 1) R = sc->Rref + sc->Eslope * (e->E - sc->Eref) / 1.0e6f;
    if (R < 0.0f) R = 0.0f;
    float z = st_normal_f(st);
    e->E += z * R * e->E / 2.35482f;
    if (sc->Sblur > 0.0f) {
        e->x += sc->Sblur * st_normal_f(st);
        e->y += sc->Sblur * st_normal_f(st);
        e->z += sc->Sblur * st_normal_f(st);
    }
}

static void blur_pulse(const or_scene* sc, dpulse_t* p)
{
    if (p->e.parn < 0) return;   /* background singles carry their own energy spread */
    stream_t st;
    st_init(&st, sc, TAG_BLUR, ((uint64_t)(uint32_t)p->e.parn << 4) | p->slot);
    blur_event(sc, &p->e, &st);
}

/* setSitenum, gPET_kernals.cu:607-640 (applied only when dlevel != 3,
 * gPET.cu:402-407; at level 3 the site set by readout is kept) */
static int32_t dead_site(const or_scene* sc, const or_event* e)
{
    switch (sc->dlevel) {
    case 0: return 0;
    case 1: return e->pann;
    case 2: return e->pann * sc->moduleN + e->modn;
    default: return e->siten;
    }
}

/* background singles (addnoise, gPET_kernals.cu:699-735, never launched by
 * the reference): a Poisson process over [t0, t1) cut into intervals, each
 * drawn from its own stream; exponential gaps of mean lambda, energy
 * N(emean, sigma), a uniform panel, module and crystal, x/y/z uniform in
 * (0, 1) as the reference leaves them, parn = eventid = -1. Time in double
 * (the reference kernel accumulates it in float). */
#define MAX_NOISE_PER_INTERVAL 4096
static int64_t noise_interval(const or_scene* sc, int64_t i, dpulse_t* out)
{
    stream_t st;
    st_init(&st, sc, TAG_NOISE, (uint64_t)i);
    double t = sc->noise_t0_us + (double)i * sc->noise_interval_us;
    double te = sc->noise_t0_us + (double)(i + 1) * sc->noise_interval_us;
    if (te > sc->noise_t1_us) te = sc->noise_t1_us;
    int64_t k = 0;
    for (; k < MAX_NOISE_PER_INTERVAL; ++k) {
        float u = st_uf(&st);
        t += (double)(-sc->noise_lambda_us * dm_logf(u));
        if (!(t < te)) break;
        if (!out) {   /* count only: skip the event's draws */
            for (int d = 0; d < 8; ++d) (void)st_uf(&st);
            continue;
        }
        dpulse_t* p = &out[k];
        memset(p, 0, sizeof(*p));
        p->e.E = sc->noise_emean + sc->noise_sigma * st_normal_f(&st);
        p->e.x = st_uf(&st); p->e.y = st_uf(&st); p->e.z = st_uf(&st);
        int pann = (int)((float)sc->npanels * st_uf(&st));
        int modn = (int)((float)sc->moduleN * st_uf(&st));
        int cryn = (int)((float)sc->crystalN * st_uf(&st));
        if (pann > sc->npanels - 1) pann = sc->npanels - 1;
        if (modn > sc->moduleN - 1) modn = sc->moduleN - 1;
        if (cryn > sc->crystalN - 1) cryn = sc->crystalN - 1;
        p->e.pann = pann; p->e.modn = modn; p->e.cryn = cryn;
        p->e.siten = pann * sc->moduleN * sc->crystalN + modn * sc->crystalN + cryn;
        p->e.parn = -1; p->e.eventid = -1; p->e.t = t;
    }
    return k;
}

static dpulse_t* add_noise(const or_scene* sc, dpulse_t* p, int64_t* n, int64_t* nnoise)
{
    *nnoise = 0;
    if (!(sc->noise_lambda_us > 0.0f) || !(sc->noise_interval_us > 0.0) || !(sc->noise_t1_us > sc->noise_t0_us))
        return p;
    const int64_t nint = (int64_t)ceil((sc->noise_t1_us - sc->noise_t0_us) / sc->noise_interval_us);
    int64_t tot = 0;
    for (int64_t i = 0; i < nint; ++i) tot += noise_interval(sc, i, NULL);
    p = (dpulse_t*)realloc(p, sizeof(dpulse_t) * (size_t)(*n + tot + 1));
    int64_t o = *n;
    for (int64_t i = 0; i < nint; ++i) o += noise_interval(sc, i, p + o);
    *nnoise = tot;
    *n += tot;
    return p;
}

static void digitize(const or_scene* sc, dpulse_t* p, int64_t n, or_result* out)
{
    /* 1. blur; 2. threshold [Eth, 2 MeV] (gPET.cu:388-396, energywindow
     * gPET_kernals.cu:641-656: dropped if E < lo or E > hi) */
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) {
        blur_pulse(sc, &p[i]);
        if (p[i].e.E < sc->Eth || p[i].e.E > 2000000.0f) continue;
        /* setSitenum overwrites the record's site (gPET_kernals.cu:607-640) */
        p[i].site = dead_site(sc, &p[i].e);
        p[i].e.siten = p[i].site;
        p[k++] = p[i];
    }
    out->n_threshold = k;
    /* 3. dead time per site in time order (orderevents detector.cu:369-385,
     * deadtime gPET_kernals.cu:657-698) with the sequential semantics the
     * reference kernel intends, in double precision: an event is lost if it
     * comes less than tau after the last event (paralyzable, type 0) or after
     * the last surviving event (non-paralyzable, type 1) of its site. */
    qsort(p, (size_t)k, sizeof(dpulse_t), cmp_site_t);
    const double tau = (double)sc->dtime_us;
    int64_t m = 0;
    double tdead = 0.0;
    for (int64_t i = 0; i < k; ++i) {
        int keep;
        if (i == 0 || p[i].site != p[i - 1].site) {
            keep = 1;
            tdead = p[i].e.t;
        } else if (p[i].e.t < tdead + tau) {
            keep = 0;
            if (sc->dtype == 0) tdead = p[i].e.t;
        } else {
            keep = 1;
            tdead = p[i].e.t;
        }
        if (keep) p[m++] = p[i];
    }
    out->n_deadtime = m;
    /* 4. energy window (gPET.cu:418-424) */
    int64_t s = 0;
    for (int64_t i = 0; i < m; ++i) {
        if (p[i].e.E < sc->ewin_lo || p[i].e.E > sc->ewin_hi) continue;
        p[s++] = p[i];
    }
    qsort(p, (size_t)s, sizeof(dpulse_t), cmp_t);
    out->n_singles = s;
    out->singles = (or_event*)malloc(sizeof(or_event) * (s ? s : 1));
    out->single_scat = (uint8_t*)malloc(s ? s : 1);
    out->single_slot = (uint8_t*)malloc(s ? s : 1);
    for (int64_t i = 0; i < s; ++i) {
        out->singles[i] = p[i].e;
        out->single_scat[i] = p[i].scat;
        out->single_slot[i] = p[i].slot;
    }
    /* 5. coincidence sorter (no counterpart in the reference): a single that
     * is not inside an open window opens [t, t+W); policy 0 keeps a window
     * holding exactly two singles in different panels, policy 1 keeps every
     * pair in different panels. Same event id and no phantom scatter -> true,
     * same event id otherwise -> scatter, different event ids -> random. */
    int64_t cap = 16, nc = 0;
    int64_t* cc = (int64_t*)malloc(sizeof(int64_t) * 2 * cap);
    uint8_t* cl = (uint8_t*)malloc(cap);
    int64_t nmult = 0;
    const double W = sc->coinc_window_us;
    for (int64_t i = 0; i < s;) {
        int64_t j = i + 1;
        while (j < s && out->singles[j].t < out->singles[i].t + W) j++;
        int64_t cnt = j - i;
        for (int64_t a = i; a < j; ++a) {
            for (int64_t b = a + 1; b < j; ++b) {
                if (sc->coinc_policy == 0 && cnt != 2) continue;
                if (out->singles[a].pann == out->singles[b].pann) continue;
                if (nc == cap) {
                    cap *= 2;
                    cc = (int64_t*)realloc(cc, sizeof(int64_t) * 2 * cap);
                    cl = (uint8_t*)realloc(cl, cap);
                }
                cc[2 * nc] = a; cc[2 * nc + 1] = b;
                uint8_t klass;
                if (out->singles[a].eventid == out->singles[b].eventid && out->singles[a].eventid >= 0)
                    klass = (out->single_scat[a] || out->single_scat[b]) ? 1 : 0;
                else
                    klass = 2;
                cl[nc] = klass;
                if (klass == 0) out->n_true++;
                else if (klass == 1) out->n_scatter++;
                else out->n_random++;
                nc++;
            }
        }
        if (cnt > 2) nmult++;
        i = j;
    }
    out->n_coinc = nc;
    out->n_multiple = nmult;
    out->coinc = cc;
    out->coinc_class = cl;
}

static int prepare(const or_scene* sc, prep_t* pp)
{
    if (sc->nmat < 1 || sc->nmat > 10 || sc->ne < 2) return -1;
    float maxden[10] = {0};
    int64_t nv = (int64_t)sc->nx * sc->ny * sc->nz;
    for (int64_t v = 0; v < nv; ++v) {
        int m = sc->mat[v];
        if (m < 0 || m >= sc->nmat) return -2;
        if (sc->den[v] > maxden[m]) maxden[m] = sc->den[v];
    }
    build_wck(sc, maxden, &pp->wph);
    float dmax[10] = {0};
    for (int i = 0; i < 2; ++i)
        if (sc->det_den[i] > dmax[sc->det_mat[i]]) dmax[sc->det_mat[i]] = sc->det_den[i];
    for (int i = 0; i < sc->nxdet; ++i)
        if (sc->xdet_den[i] > dmax[sc->xdet_mat[i]]) dmax[sc->xdet_mat[i]] = sc->xdet_den[i];
    build_wck(sc, dmax, &pp->wdet);
    if (sc->nsrc > 64) return -3;
    for (int i = 0; i < sc->nsrc; ++i) {
        double th = (double)sc->iso_halftime[sc->src_type[i]];
        double tau = th / 0.69314718055994530942;
        pp->ntau_us[i] = -tau * 1e6;
        pp->cfac[i] = -expm1(-sc->dt_s / tau);
    }
    return 0;
}

int oracle_run(const or_scene* sc, int64_t d_begin, int64_t d_end, int nthreads, int flags, or_result* out)
{
    memset(out, 0, sizeof(*out));
    prep_t* pp = (prep_t*)malloc(sizeof(prep_t));
    int rc = prepare(sc, pp);
    if (rc) { free(pp); return rc; }
    int64_t nd = d_end - d_begin;
    if (nd < 0) { free(pp); return -4; }
    out->n_decays = nd;
    if (flags & 1) out->exits = (or_exit*)calloc((size_t)(2 * nd + 1), sizeof(or_exit));
    if (flags & 4) out->source = (or_src*)calloc((size_t)(2 * nd + 1), sizeof(or_src));
#ifdef _OPENMP
    if (nthreads < 1) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    tbuf_t* tb = (tbuf_t*)calloc((size_t)nthreads, sizeof(tbuf_t));
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
#ifdef _OPENMP
        int tid = omp_get_thread_num();
#else
        int tid = 0;
#endif
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t d = d_begin; d < d_end; ++d)
            simulate_decay(sc, pp, d, out->exits ? out->exits + 2 * (d - d_begin) : NULL,
                           out->source ? out->source + 2 * (d - d_begin) : NULL, &tb[tid], flags);
    }
    int64_t np = 0, nh = 0;
    for (int t = 0; t < nthreads; ++t) {
        np += tb[t].n; nh += tb[t].nh;
        out->n_entered += tb[t].n_entered; out->n_pairs += tb[t].n_pairs;
        out->n_overflow += tb[t].n_overflow; out->n_stepcap += tb[t].n_stepcap;
    }
    dpulse_t* p = (dpulse_t*)malloc(sizeof(dpulse_t) * (np ? np : 1));
    out->hit_id = (int32_t*)malloc(sizeof(int32_t) * 5 * (nh ? nh : 1));
    out->hit_f = (float*)malloc(sizeof(float) * 5 * (nh ? nh : 1));
    int64_t o = 0, oh = 0;
    for (int t = 0; t < nthreads; ++t) {
        for (int64_t i = 0; i < tb[t].n; ++i, ++o) {
            p[o].e = tb[t].ev[i]; p[o].scat = tb[t].scat[i]; p[o].slot = tb[t].slot[i]; p[o].site = 0;
        }
        if (tb[t].nh) {
            memcpy(out->hit_id + 5 * oh, tb[t].hid, sizeof(int32_t) * 5 * tb[t].nh);
            memcpy(out->hit_f + 5 * oh, tb[t].hf, sizeof(float) * 5 * tb[t].nh);
            oh += tb[t].nh;
        }
        free(tb[t].ev); free(tb[t].scat); free(tb[t].slot); free(tb[t].hid); free(tb[t].hf);
    }
    free(tb);
    out->n_hits = nh;
    qsort(p, (size_t)np, sizeof(dpulse_t), cmp_parn_slot);
    out->n_pulses = np;
    out->pulses = (or_event*)malloc(sizeof(or_event) * (np ? np : 1));
    out->pulse_scat = (uint8_t*)malloc(np ? np : 1);
    out->pulse_slot = (uint8_t*)malloc(np ? np : 1);
    for (int64_t i = 0; i < np; ++i) {
        out->pulses[i] = p[i].e; out->pulse_scat[i] = p[i].scat; out->pulse_slot[i] = p[i].slot;
    }
    p = add_noise(sc, p, &np, &out->n_noise);
    digitize(sc, p, np, out);
    free(p);
    free(pp);
    return 0;
}

int oracle_digitize(const or_scene* sc, const or_event* pulses, const uint8_t* scat, const uint8_t* slot,
                    int64_t n, or_result* out)
{
    memset(out, 0, sizeof(*out));
    dpulse_t* p = (dpulse_t*)malloc(sizeof(dpulse_t) * (n ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        p[i].e = pulses[i]; p[i].scat = scat[i]; p[i].slot = slot[i]; p[i].site = 0;
    }
    out->n_pulses = n;
    p = add_noise(sc, p, &n, &out->n_noise);
    digitize(sc, p, n, out);
    free(p);
    return 0;
}

void oracle_free_result(or_result* r)
{
    free(r->exits); free(r->source); free(r->pulses); free(r->pulse_scat); free(r->pulse_slot);
    free(r->hit_id); free(r->hit_f); free(r->singles); free(r->single_scat); free(r->single_slot);
    free(r->coinc); free(r->coinc_class);
    memset(r, 0, sizeof(*r));
}

/* ------------------------------------------------ known-answer test hooks */
static void hook_scene(or_scene* sc, uint64_t seed)
{
    memset(sc, 0, sizeof(*sc));
    sc->seed = seed;
}

/* positron kinetic energies (eV) from sampleEkPositron for one isotope row */
void oracle_sample_ek(const float* coef8, uint64_t seed, int64_t n, double* out)
{
    or_scene sc;
    hook_scene(&sc, seed);
    for (int64_t i = 0; i < n; ++i) {
        stream_t st;
        st_init(&st, &sc, TAG_DECAY, (uint64_t)i);
        or_scene s2 = sc;
        s2.iso_coef = coef8;
        out[i] = (double)sample_ek(&s2, 0, &st);
    }
}

/* Klein-Nishina (free electron) samples: cos(theta) and energy fraction */
void oracle_kn_sample(double energy, uint64_t seed, int64_t n, double* cost, double* efrac)
{
    or_scene sc;
    hook_scene(&sc, seed);
    for (int64_t i = 0; i < n; ++i) {
        stream_t st;
        st_init(&st, &sc, TAG_DET, (uint64_t)i);
        real ef, c;
        kn_sample((real)energy, &st, &ef, &c);
        cost[i] = (double)c;
        efrac[i] = (double)ef;
    }
}

/* annihilation pairs: angle between the two photons (rad) and their energies */
void oracle_pair_angles(float sigma, uint64_t seed, int64_t n, double* angle, double* e0, double* e1)
{
    or_scene sc;
    hook_scene(&sc, seed);
    sc.noncol_sigma = sigma;
    real pos[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; ++i) {
        stream_t st;
        st_init(&st, &sc, TAG_DECAY, (uint64_t)i);
        photon_t ph[2];
        make_pair(&sc, &st, pos, ph, 0.0, NULL);
        double d = (double)ph[0].u[0] * ph[1].u[0] + (double)ph[0].u[1] * ph[1].u[1] + (double)ph[0].u[2] * ph[1].u[2];
        double n0 = sqrt((double)ph[0].u[0] * ph[0].u[0] + (double)ph[0].u[1] * ph[0].u[1] + (double)ph[0].u[2] * ph[0].u[2]);
        double n1 = sqrt((double)ph[1].u[0] * ph[1].u[0] + (double)ph[1].u[1] * ph[1].u[1] + (double)ph[1].u[2] * ph[1].u[2]);
        d /= n0 * n1;
        if (d > 1) d = 1;
        if (d < -1) d = -1;
        angle[i] = acos(d);
        e0[i] = (double)ph[0].E;
        e1[i] = (double)ph[1].E;
    }
}

/* deterministic math of detmath.h, for accuracy tests:
 * which 0 logf, 1 expf, 2 sin(2 pi x), 3 cos(2 pi x), 4 cbrtf */
void oracle_detmath(int which, int64_t n, const float* x, float* y)
{
    for (int64_t i = 0; i < n; ++i) {
        float s, c;
        switch (which) {
        case 0: y[i] = dm_logf(x[i]); break;
        case 1: y[i] = dm_expf(x[i]); break;
        case 2: dm_sincos_turns(x[i], &s, &c); y[i] = s; break;
        case 3: dm_sincos_turns(x[i], &s, &c); y[i] = c; break;
        default: y[i] = dm_cbrtf(x[i]); break;
        }
    }
}

void oracle_detmath_log(int64_t n, const double* x, double* y)
{
    for (int64_t i = 0; i < n; ++i) y[i] = dm_log(x[i]);
}

/* which 0: dm_log1p_small, 1: dm_u01d of (hi, lo) given as x = hi * 2^32 + lo */
void oracle_detmath_d(int which, int64_t n, const double* x, double* y)
{
    for (int64_t i = 0; i < n; ++i) {
        if (which == 0) {
            y[i] = dm_log1p_small(x[i]);
        } else {
            const uint64_t v = (uint64_t)x[i];
            y[i] = dm_u01d((uint32_t)(v >> 32), (uint32_t)v);
        }
    }
}

#ifdef ORACLE_TAPE
/* ------------------------------------------------------------------------
 * Tape-driven entry points: each runs one step of the oracle on random words
 * given by the caller instead of its Philox streams, so the pins in tests/
 * can feed the oracle and the reference's own functions (built for the CPU)
 * exactly the same words and compare what they compute. */
static void st_tape(stream_t* s, const uint32_t* tape, int64_t n)
{
    memset(s, 0, sizeof(*s));
    s->tape = tape;
    s->tape_n = n;
    s->tape_pos = 0;
}

static void photon_from(photon_t* p, const float in[7], double t_us)
{
    memset(p, 0, sizeof(*p));
    for (int k = 0; k < 3; ++k) { p->x[k] = (real)in[k]; p->u[k] = (real)in[3 + k]; }
    p->E = (real)in[6];
    p->t = t_us;
}

/* photon(), gPET_kernals.cu:256-345, with the majorant table given */
int oracle_tape_phantom(const or_scene* sc, const float* wtab, float e0, float ide, const float in[7], double t_us,
                        const uint32_t* tape, int64_t n, double out[7], double* t_out, int32_t* nscat, int64_t* used)
{
    static wck_t w;
    w.e0 = e0; w.ide = ide;
    memcpy(w.tab, wtab, sizeof(w.tab));
    photon_t p;
    photon_from(&p, in, t_us);
    stream_t st;
    st_tape(&st, tape, n);
    int status = phantom_transport(sc, &w, &p, &st);
    for (int k = 0; k < 3; ++k) { out[k] = (double)p.x[k]; out[3 + k] = (double)p.u[k]; }
    out[6] = (double)p.E;
    *t_out = p.t + (double)p.tf;
    *nscat = p.nscat;
    *used = st.tape_pos;
    return status;
}

/* photonde per photon, gPET_kernals.cu:839-1233: panel search, detector
 * transport with the detector majorant given, adder, readout; pulses (parn 0)
 * into out[cap]; returns the pulse count, *panel the entered panel or -1 */
int oracle_tape_detector(const or_scene* sc, const float* wtab, float e0, float ide, const float in[7], double t_us,
                         int32_t eventid, const uint32_t* tape, int64_t n, or_event* out, int cap, int32_t* panel,
                         int64_t* used)
{
    static wck_t w;
    w.e0 = e0; w.ide = ide;
    memcpy(w.tab, wtab, sizeof(w.tab));
    photon_t p;
    photon_from(&p, in, t_us);
    local_t q;
    *panel = -1;
    *used = 0;
    if (!enter_panel(sc, &p, &q)) return 0;
    *panel = q.panel;
    stream_t st;
    st_tape(&st, tape, n);
    tbuf_t tb;
    memset(&tb, 0, sizeof(tb));
    detector_transport(sc, &w, &q, 0, eventid, 0, &st, &tb, 0);
    *used = st.tape_pos;
    int k = (int)tb.n;
    for (int i = 0; i < k && i < cap; ++i) out[i] = tb.ev[i];
    free(tb.ev); free(tb.scat); free(tb.slot); free(tb.hid); free(tb.hf);
    return k;
}

/* comsam, free-electron Klein-Nishina (gPET_kernals.cu:90-126) */
void oracle_tape_kn(double e, const uint32_t* tape, int64_t n, double* efrac, double* cost, int64_t* used)
{
    stream_t st;
    st_tape(&st, tape, n);
    real ef, c;
    kn_sample((real)e, &st, &ef, &c);
    *efrac = (double)ef; *cost = (double)c; *used = st.tape_pos;
}

/* comsam from the surface (which 0) and rylsam (which 1), gPET_kernals.cu:66-88, 128-146 */
void oracle_tape_surface(const or_scene* sc, int which, double e, int m, const uint32_t* tape, int64_t n,
                         double* efrac, double* cost, int64_t* used)
{
    stream_t st;
    st_tape(&st, tape, n);
    real ef = (real)1.0, c;
    if (which == 0) compton_surface(sc, (real)e, m, &st, &ef, &c);
    else c = rayleigh_surface(sc, (real)e, m, &st);
    *efrac = (double)ef; *cost = (double)c; *used = st.tape_pos;
}

/* sampleEkPositron (gPET_kernals.cu:420-443) for one isotope's coefficients */
double oracle_tape_sample_ek(const float coef8[8], const uint32_t* tape, int64_t n, int64_t* used)
{
    or_scene sc;
    memset(&sc, 0, sizeof(sc));
    sc.iso_coef = coef8;
    stream_t st;
    st_tape(&st, tape, n);
    double ek = (double)sample_ek(&sc, 0, &st);
    *used = st.tape_pos;
    return ek;
}

/* getPositionFromShape (gPET_kernals.cu:445-482) */
void oracle_tape_shape(int shape, const float coef6[6], const uint32_t* tape, int64_t n, double p[3], int64_t* used)
{
    or_scene sc;
    memset(&sc, 0, sizeof(sc));
    int32_t sh = shape;
    sc.src_coef = coef6;
    sc.src_shape = &sh;
    stream_t st;
    st_tape(&st, tape, n);
    real r[3];
    shape_position(&sc, 0, &st, r);
    p[0] = (double)r[0]; p[1] = (double)r[1]; p[2] = (double)r[2];
    *used = st.tape_pos;
}

/* setPositronRange (gPET_kernals.cu:347-418) in the scene's phantom; dir NULL:
 * the sampled direction (usedirection 0) */
void oracle_tape_positron_range(const or_scene* sc, const float x[3], double ek, const float* dir,
                                const uint32_t* tape, int64_t n, double out[3], int64_t* used)
{
    stream_t st;
    st_tape(&st, tape, n);
    real p[3] = {(real)x[0], (real)x[1], (real)x[2]};
    real d[3];
    if (dir) { d[0] = (real)dir[0]; d[1] = (real)dir[1]; d[2] = (real)dir[2]; }
    positron_range(sc, p, (real)ek, dir ? d : NULL, &st, NULL);
    out[0] = (double)p[0]; out[1] = (double)p[1]; out[2] = (double)p[2];
    *used = st.tape_pos;
}

/* setPositionForPhoton (gPET_kernals.cu:563-604) for one positron record:
 * out = position (3), photon 0 direction and energy (4), photon 1 (4) */
void oracle_tape_psf_pair(const or_scene* sc, const float x[3], const float v4[4], int useprange,
                          const uint32_t* tape, int64_t n, double out[11], int64_t* used)
{
    stream_t st;
    st_tape(&st, tape, n);
    real pos[3] = {(real)x[0], (real)x[1], (real)x[2]};
    real dir[3] = {(real)v4[0], (real)v4[1], (real)v4[2]};
    real spare = (real)0.0;
    if (useprange) positron_range(sc, pos, (real)v4[3], dir, &st, &spare);
    photon_t ph[2];
    make_pair(sc, &st, pos, ph, 1.0, useprange ? &spare : NULL);
    for (int k = 0; k < 3; ++k) out[k] = (double)pos[k];
    for (int j = 0; j < 2; ++j) {
        for (int k = 0; k < 3; ++k) out[3 + 4 * j + k] = (double)ph[j].u[k];
        out[6 + 4 * j] = (double)ph[j].E;
    }
    *used = st.tape_pos;
}

/* crystalSearch (gPET_kernals.cu:1236-1279) in panel p of the scene */
void oracle_crystal_search_at(const or_scene* sc, int p, const double x[3], int32_t ids[3])
{
    real r[3] = {(real)x[0], (real)x[1], (real)x[2]};
    int m = -1, M = -1, L = -1;
    crystal_search(sc, sc->panels + (size_t)p * OR_PANEL_STRIDE, r, &m, &M, &L);
    ids[0] = m; ids[1] = M; ids[2] = L;
}

/* adder over n deposits of one photon, then readout (gPET_kernals.cu:737-813) */
int oracle_adder_readout(const or_scene* sc, const or_event* dep, int n, or_event* out, int cap)
{
    or_event ev[MAX_PULSE];
    int nev = 0;
    for (int i = 0; i < n; ++i)
        if (!adder(ev, &nev, &dep[i])) return -1;
    or_event tmp[MAX_PULSE];
    int k = readout(sc, ev, nev, tmp);
    for (int i = 0; i < k && i < cap; ++i) out[i] = tmp[i];
    return k;
}

/* the Woodcock majorant the oracle builds for the scene (which 0 phantom,
 * 1 detector): 4096 mean free paths, first energy, inverse spacing */
int oracle_majorant(const or_scene* sc, int which, float* tab, float* e0, float* ide)
{
    static prep_t pp;
    int rc = prepare(sc, &pp);
    if (rc) return rc;
    const wck_t* w = which == 0 ? &pp.wph : &pp.wdet;
    memcpy(tab, w->tab, sizeof(w->tab));
    *e0 = w->e0;
    *ide = w->ide;
    return 0;
}

/* blur (gPET_kernals.cu:814-837) of one pulse */
void oracle_tape_blur(const or_scene* sc, or_event* e, const uint32_t* tape, int64_t n, int64_t* used)
{
    stream_t st;
    st_tape(&st, tape, n);
    blur_event(sc, e, &st);
    *used = st.tape_pos;
}
#endif /* ORACLE_TAPE */
