// device.cuh - scene descriptor, counter-based RNG streams and the photon
// physics of the gPET hot path, for sm_103a.
//
// Every floating-point expression here is written in the same order as the
// single-precision build of the CPU oracle, and the translation units are
// compiled with -fmad=false, so a history computed here matches the oracle's
// FP32 build bit for bit (fused steps appear only as explicit fma in
// detmath.h). Reference: gPET_kernals.cu (file:line at each function).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include "detmath.h"

namespace gpet {

constexpr int kPanelStride = 32;
constexpr int kMaxPanels = 256;
constexpr int kMaxSurf = 5;
constexpr int kMaxSrc = 64;
constexpr int kMaxPulse = 8;     // distinct crystals per photon (adder list)
constexpr int kMaxHits = 16;     // deposits recorded per photon
constexpr int kMaxSteps = 100000;
constexpr int kNwck = 4096;
constexpr float kMC2 = 510999.1f;              // constants.h:37
constexpr float kIMC2 = 1.95695060911e-6f;     // constants.h:38
constexpr double kSpe = 29979.2458;            // cm/us, gPET_kernals.cu:264

enum : uint32_t { kTagDecay = 1, kTagPhantom = 2, kTagDet = 4, kTagBlur = 8, kTagNoise = 9 };

// Everything one simulation needs on the device. Lives in device memory; the
// kernels copy it into shared memory once per block.
struct SimDesc {
    uint32_t key0, key1;
    // cross sections on one energy grid: xs4[m*ne + i] = (lamph, compt, rayle, phote)
    int32_t nmat, ne;
    float e0, idle;
    const float4* xs4;
    int32_t ncp_c, ne_c;
    float idcp_c, ide_c;
    const float* cmpsf;           // [nmat][ncp_c][ne_c]
    int32_t ncp_r, ne_r;
    float idcp_r, ide_r;
    const float* rayff;
    float wck_e0, wck_ide;
    const float* wck_ph;          // [4096]
    const float* wck_det;         // [4096]
    // phantom: vox[i] = (density bits, material), x fastest; or, with vox16
    // set, vox[vox16[i]] (a palette of the distinct pairs)
    int32_t nx, ny, nz;
    float dx, dy, dz, idx, idy, idz, offx, offy, offz;
    const uint2* vox;
    const uint16_t* vox16;
    // radius of uniform density around each voxel (prange_uniform), or null
    const int8_t* prmap;
    // the uploaded densities, one float per voxel (the bits the palette
    // holds), for the positron range's lookups where they fit in L2; or null
    const float* den;
    float prdmin;                 // min(dx, dy, dz)
    // detector
    int32_t npanels;
    const float* panels;          // [npanels][32]
    int32_t ndetmat;              // 0 crystal, 1 gap, 2.. crystal regions of surfaces 0..
    int32_t det_mat[8];
    float det_den[8];
    int32_t moduleN, crystalN, moduleNy, crystalNy;
    int32_t nsurface;
    float surface[10 * kMaxSurf];
    float eabsph;
    int32_t rdepth, rpolicy;
    // bound of the panel entry faces for a quick rejection (see
    // may_reach_panels): faces parallel to the z axis, none closer to it than
    // sqrt(ring_rin2), all within [ring_zmin, ring_zmax] (padded); 0 none,
    // 1 the bound, 2 the bound and every face entered only from the axis side
    int32_t ring_test;
    float ring_zmin, ring_zmax, ring_rin2;
    // sources (last: the transport kernels stage only the fields before
    // them, kSimTransportBytes, in shared memory)
    int32_t nsrc;
    int64_t src_end[kMaxSrc];     // exclusive end of each source's decay range
    int32_t src_type[kMaxSrc], src_shape[kMaxSrc];
    float src_coef[kMaxSrc][6];
    double src_ntau_us[kMaxSrc], src_cfac[kMaxSrc];   // -lifetime (us), 1 - exp(-window / lifetime)
    float iso_ratio[kMaxSrc];     // indexed by source (ratio of its isotope)
    float iso_coef[kMaxSrc][8];   // indexed by source
    double tstart_us;
    int32_t useprange;
    float noncol_sigma;
    int64_t npsf;
    const double* psf;            // [npsf][8]
    int32_t psf_ptype;
    int32_t pad_;
};

// bytes of a SimDesc the phantom and detector kernels use (everything before
// the sources)
constexpr size_t kSimTransportBytes = offsetof(SimDesc, nsrc);
static_assert(kSimTransportBytes % 4 == 0, "staged as 32-bit words");

// ------------------------------------------------------------------ RNG
// A stream is keyed by (key, tag, 64-bit id): its state is the Philox4x32-10
// block (Salmon et al., SC'11) of counter (0, tag, id) under the key, and its
// words come from xoshiro128** (Blackman & Vigna, "Scrambled linear
// pseudorandom number generators", ACM TOMS 2021) run from that state. The
// counter-based seed keeps every decay's, photon's and pulse's draws
// independent of which thread takes it and when; the sequential generator
// costs a fraction of a Philox block per word.
struct Stream {
    uint32_t s[4];
};

__device__ __forceinline__ void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                         uint32_t k1, uint32_t out[4])
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// state of stream (key k0 k1, tag, id hi:lo); the all-zero state, which
// xoshiro never leaves, is replaced by a fixed one
__device__ __forceinline__ void st_seed(uint32_t (&s)[4], uint32_t k0, uint32_t k1, uint32_t tag, uint32_t idlo,
                                        uint32_t idhi)
{
    philox10(0u, tag, idlo, idhi, k0, k1, s);
    if ((s[0] | s[1] | s[2] | s[3]) == 0u) s[0] = 0x9E3779B9u;
}

// next word of xoshiro128**: rotl(s1 * 5, 7) * 9, then the linear step
__device__ __forceinline__ uint32_t xo_next(uint32_t (&s)[4])
{
    const uint32_t m = s[1] * 5u;
    const uint32_t v = __funnelshift_l(m, m, 7) * 9u;
    const uint32_t t = s[1] << 9;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = __funnelshift_l(s[3], s[3], 11);
    return v;
}

__device__ __forceinline__ void st_init(Stream& s, uint32_t k0, uint32_t k1, uint32_t tag, uint64_t id)
{
    st_seed(s.s, k0, k1, tag, (uint32_t)id, (uint32_t)(id >> 32));
}

__device__ __forceinline__ uint32_t st_next(Stream& s) { return xo_next(s.s); }

__device__ __forceinline__ float st_u(Stream& s) { return dm_u01(st_next(s)); }

__device__ __forceinline__ double st_ud(Stream& s)
{
    uint32_t hi = st_next(s);
    uint32_t lo = st_next(s);
    return dm_u01d(hi, lo);
}

__device__ __forceinline__ float st_normal(Stream& s)
{
    float u1 = st_u(s);
    float u2 = st_u(s);
    return dm_normal(u1, u2);
}

__device__ __forceinline__ void st_normal2(Stream& s, float& n1, float& n2)
{
    float u1 = st_u(s);
    float u2 = st_u(s);
    dm_normal2(u1, u2, &n1, &n2);
}

// ---------------------------------------------------------------- lookups
// value of a linearly filtered 1-D table at fractional index x, edges clamped
// (the reference's tex1D lookups, gPET_kernals.cu:31-64)
__device__ __forceinline__ float lerp1(const float* __restrict__ tab, int n, float x)
{
    if (!(x > 0.0f)) return __ldg(tab);
    if (x >= (float)(n - 1)) return __ldg(tab + n - 1);
    int i = (int)x;
    float f = x - (float)i;
    float a = __ldg(tab + i), b = __ldg(tab + i + 1);
    return dm_fma(f, b - a, a);
}

// all four cross sections of material m at energy e
__device__ __forceinline__ float4 xs_at(const SimDesc& S, int m, float e)
{
    float x = S.idle * (e - S.e0);
    const float4* t = S.xs4 + (size_t)m * S.ne;
    int n = S.ne;
    if (!(x > 0.0f)) return __ldg(t);
    if (x >= (float)(n - 1)) return __ldg(t + n - 1);
    int i = (int)x;
    float f = x - (float)i;
    float4 a = __ldg(t + i), b = __ldg(t + i + 1);
    float4 r;
    r.x = dm_fma(f, b.x - a.x, a.x);
    r.y = dm_fma(f, b.y - a.y, a.y);
    r.z = dm_fma(f, b.z - a.z, a.z);
    r.w = dm_fma(f, b.w - a.w, a.w);
    return r;
}

// bilinear inverse-CDF surface lookup, clamped (tex3D of s_tex / f_tex,
// gPET_kernals.cu:82, 142)
__device__ __forceinline__ float lerp2(const float* __restrict__ s, int ncp, int ne, float xe, float ycp)
{
    if (!(xe > 0.0f)) xe = 0.0f;
    if (xe > (float)(ne - 1)) xe = (float)(ne - 1);
    if (!(ycp > 0.0f)) ycp = 0.0f;
    if (ycp > (float)(ncp - 1)) ycp = (float)(ncp - 1);
    int ie = (int)xe; if (ie > ne - 2) ie = ne - 2;
    int ic = (int)ycp; if (ic > ncp - 2) ic = ncp - 2;
    float fe = xe - (float)ie, fc = ycp - (float)ic;
    const float* r0 = s + (size_t)ic * ne;
    const float* r1 = r0 + ne;
    float a00 = __ldg(r0 + ie), a01 = __ldg(r0 + ie + 1), a10 = __ldg(r1 + ie), a11 = __ldg(r1 + ie + 1);
    float a = dm_fma(fe, a01 - a00, a00);
    float b = dm_fma(fe, a11 - a10, a10);
    return dm_fma(fc, b - a, a);
}

__device__ __forceinline__ float wck_at(const float* __restrict__ tab, float e0, float ide, float e)
{
    return lerp1(tab, kNwck, ide * (e - e0));
}

// ---------------------------------------------------------------- geometry
// rotate(), gPET_kernals.cu:172-254; azimuth given in turns
__device__ __forceinline__ void rotate(float& u, float& v, float& w, float costh, float phi_turns)
{
    float rho2 = u * u + v * v;
    float norm = rho2 + w * w;
    if (fabsf(norm - 1.0f) > 1.0e-4f) {
        norm = 1.0f / dm_sqrt(norm);
        u = u * norm; v = v * norm; w = w * norm;
    }
    float sinphi, cosphi;
    dm_sincos_turns(phi_turns, &sinphi, &cosphi);
    float temp = costh * costh;
    if (rho2 > 1.0e-20f) {
        float sthrho = temp < 1.0f ? dm_sqrt((1.0f - temp) / rho2) : 0.0f;
        float urho = u * sthrho, vrho = v * sthrho;
        float uu = u * costh - vrho * sinphi + w * urho * cosphi;
        float vv = v * costh + urho * sinphi + w * vrho * cosphi;
        float ww = w * costh - rho2 * sthrho * cosphi;
        u = uu; v = vv; w = ww;
    } else {
        float sinth = temp < 1.0f ? dm_sqrt(1.0f - temp) : 0.0f;
        v = sinth * sinphi;
        if (w > 0.0f) { u = sinth * cosphi; w = costh; }
        else { u = -sinth * cosphi; w = -costh; }
    }
}

// getAbsVox, gPET_kernals.cu:19-29 (index 0 counts as outside)
__device__ __forceinline__ bool abs_vox(const SimDesc& S, float x, float y, float z, int& ix, int& iy, int& iz)
{
    float vx = (x - S.offx) * S.idx;
    float vy = (y - S.offy) * S.idy;
    float vz = (z - S.offz) * S.idz;
    bool in = vx >= 1.0f && vx < (float)S.nx && vy >= 1.0f && vy < (float)S.ny && vz >= 1.0f && vz < (float)S.nz;
    if (in) { ix = (int)vx; iy = (int)vy; iz = (int)vz; }
    return in;
}

// (ix, iy, iz) in range; a phantom holds fewer than 2^31 voxels
__device__ __forceinline__ uint2 voxel(const SimDesc& S, int ix, int iy, int iz)
{
    const uint32_t i = (uint32_t)ix + (uint32_t)S.nx * ((uint32_t)iy + (uint32_t)S.ny * (uint32_t)iz);
    if (S.vox16) return __ldg(S.vox + __ldg(S.vox16 + i));
    return __ldg(S.vox + i);
}

// density of voxel (ix, iy, iz) (in range): one load from the density array
// where there is one, else through the phantom's voxel records
__device__ __forceinline__ float den_at(const SimDesc& S, int ix, int iy, int iz)
{
    if (S.den) return __ldg(S.den + ((uint32_t)ix + (uint32_t)S.nx * ((uint32_t)iy + (uint32_t)S.ny * (uint32_t)iz)));
    return __uint_as_float(voxel(S, ix, iy, iz).x);
}

__device__ __forceinline__ float den_clamped(const SimDesc& S, int ix, int iy, int iz)
{
    ix = ix < 0 ? 0 : (ix > S.nx - 1 ? S.nx - 1 : ix);
    iy = iy < 0 ? 0 : (iy > S.ny - 1 ? S.ny - 1 : iy);
    iz = iz < 0 ? 0 : (iz > S.nz - 1 ? S.nz - 1 : iz);
    return den_at(S, ix, iy, iz);
}

// ---------------------------------------------------------------- source
// getPositionFromShape, gPET_kernals.cu:445-482
__device__ __forceinline__ void shape_position(const SimDesc& S, int si, Stream& st, float p[3])
{
    const float* c = S.src_coef[si];
    int shape = S.src_shape[si];
    if (shape < 0 || shape > 2) shape = 0;
    if (shape == 0) {
        float a = st_u(st), b = st_u(st), d = st_u(st);
        p[0] = c[0] + c[3] * (-1.0f + 2.0f * a) * 0.5f;
        p[1] = c[1] + c[4] * (-1.0f + 2.0f * b) * 0.5f;
        p[2] = c[2] + c[5] * (-1.0f + 2.0f * d) * 0.5f;
    } else if (shape == 1) {
        float phi = st_u(st);
        float r = c[3] * dm_sqrt(st_u(st));
        float zz = st_u(st);
        float s, cs;
        dm_sincos_turns(phi, &s, &cs);
        p[0] = c[0] + r * cs;
        p[1] = c[1] + r * s;
        p[2] = c[2] + c[4] * (-1.0f + 2.0f * zz) * 0.5f;
    } else {
        float phi = st_u(st);
        float cost = -1.0f + 2.0f * st_u(st);
        float r = c[3] * dm_cbrtf(st_u(st));
        float s, cs;
        dm_sincos_turns(phi, &s, &cs);
        float st2 = dm_sqrt(1.0f - cost * cost);
        p[0] = c[0] + r * st2 * cs;
        p[1] = c[1] + r * st2 * s;
        p[2] = c[2] + r * cost;
    }
}

// sampleEkPositron, gPET_kernals.cu:420-443 (kinetic energy, eV)
__device__ __forceinline__ float sample_ek(const float* cf, Stream& st)
{
    float e = 0.0f;
    for (int it = 0; it < 100000; ++it) {
        e = st_u(st) * (cf[0] - 0.511f) + 0.511f;
        float u = cf[1] * st_u(st);
        float sum = cf[2];
#pragma unroll
        for (int k = 3; k < 8; ++k) sum = sum * e + cf[k];
        if (!(u > sum)) break;
    }
    return (e - 0.511f) * 1.0e6f;
}

// setPositronRange, gPET_kernals.cu:347-418, in three parts: the Gaussian
// displacement (prange_draw), the closed form for a walk that stays in voxels
// of one density (prange_uniform) and the voxel walk itself (prange_walk_*,
// density read from the voxel being entered; outside the phantom the
// remaining range is walked in air). The walk draws no random numbers, so
// k_source can leave it to k_walk and go on with the pair emission.
constexpr int kPrMax = 6;        // largest radius the uniform-density map holds

// displacement d (length r, returned) of a positron of kinetic energy ek (eV);
// along dir when given. spare (may be null): the second normal of the last
// Box-Muller pair, which the pair emission uses for its non-collinearity angle
__device__ __forceinline__ float prange_draw(float ek, const float* dir, Stream& st, float d[3], float* spare)
{
    float ekin = ek / 1.0e6f;
    const float b1 = 5.44040782f, b2 = 0.369516529f;
    float rex = 0.1f * b1 * ekin * ekin / (b2 + ekin);
    float sigma = rex / 2.0f;
    {
        float n1, n2;
        st_normal2(st, n1, n2);
        d[0] = sigma * n1;
        d[1] = sigma * n2;
        float n3, n4;
        st_normal2(st, n3, n4);
        d[2] = sigma * n3;
        if (spare) *spare = n4;
    }
    float r = dm_sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (dir) {
        float tmp = dm_sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        d[0] = r * dir[0] / tmp; d[1] = r * dir[1] / tmp; d[2] = r * dir[2] / tmp;
    }
    return r;
}

// The walk ends where the density-weighted path length reaches r. Where every
// voxel it reads has the density rho, that is x + (r / rho) * d / r exactly.
// The voxels it reads lie within floor(L / dmin) + 2 voxels (Chebyshev) of the
// start voxel, L = r / rho (the end voxel, plus the voxel entered beyond it);
// prmap[v] = R says that all voxels within R of v have v's density and lie in
// [1, n-2] on every axis, so L < (R - 1.5) * dmin (half a voxel of margin)
// keeps the walk inside. Returns false where the walk is needed. A walk that
// reaches beyond the uniform cube (R >= 2) starts where its first
// lim = (R - 1.5) * dmin of path would take it: x moves by lim along d / r and
// *s0 = lim * rho is the density-weighted length already covered (the walk
// would read only voxels of density rho up to there: the voxel holding that
// point lies within R - 1 of the start voxel, and the one entered after it
// within R); otherwise x is unchanged and *s0 = 0. est = about the number of
// voxel faces the rest of the walk crosses at the start voxel's density (0
// outside the phantom, where it takes one step). A zero displacement moves
// nothing, as in the walk.
__device__ __forceinline__ bool prange_uniform(const SimDesc& S, float x[3], const float d[3], float r, float& est,
                                               float& s0)
{
    est = 0.0f;
    s0 = 0.0f;
    if (!(r > 0.0f)) return true;
    int ix, iy, iz;
    if (!abs_vox(S, x[0], x[1], x[2], ix, iy, iz)) return false;
    const uint32_t i = (uint32_t)ix + (uint32_t)S.nx * ((uint32_t)iy + (uint32_t)S.ny * (uint32_t)iz);
    const int R = S.prmap ? __ldg(S.prmap + i) : 0;
    const float rho = den_at(S, ix, iy, iz);
    if (!(rho > 0.0f)) {
        est = 1.0e30f;
        return false;
    }
    const float L = r / rho;
    const float sum_d = fabsf(d[0]) + fabsf(d[1]) + fabsf(d[2]);
    if (R < 2) {
        est = sum_d / (rho * S.prdmin);
        return false;
    }
    const float lim = ((float)R - 1.5f) * S.prdmin;
    const float ir = 1.0f / r;
    const float dn0 = d[0] * ir, dn1 = d[1] * ir, dn2 = d[2] * ir;
    if (L < lim) {
        x[0] = x[0] + L * dn0;
        x[1] = x[1] + L * dn1;
        x[2] = x[2] + L * dn2;
        return true;
    }
    x[0] = x[0] + lim * dn0;
    x[1] = x[1] + lim * dn1;
    x[2] = x[2] + lim * dn2;
    s0 = lim * rho;
    est = (L - lim) * ir * sum_d / S.prdmin;
    return false;
}

// state of one voxel walk
struct PWalk {
    float x[3], id[3], dn[3], r, s;
    float xmax, ymax, zmax;       // far faces of the phantom
    int v[3];
    int guard;
    int pos;                      // bit k: d[k] > 0
    bool inside;
};

// set up the walk of displacement d (length r) from x, with the
// density-weighted length s0 already covered; false if it has no step
__device__ __forceinline__ bool prange_walk_init(const SimDesc& S, PWalk& w, const float x[3], const float d[3],
                                                 float r, float s0)
{
    // reciprocals once: the walk multiplies instead of dividing
    w.id[0] = 1.0f / d[0]; w.id[1] = 1.0f / d[1]; w.id[2] = 1.0f / d[2];
    const float ir = 1.0f / r;
    w.dn[0] = d[0] * ir; w.dn[1] = d[1] * ir; w.dn[2] = d[2] * ir;
    w.pos = (d[0] > 0.0f ? 1 : 0) | (d[1] > 0.0f ? 2 : 0) | (d[2] > 0.0f ? 4 : 0);
    w.x[0] = x[0]; w.x[1] = x[1]; w.x[2] = x[2];
    w.xmax = S.offx + (float)S.nx * S.dx;
    w.ymax = S.offy + (float)S.ny * S.dy;
    w.zmax = S.offz + (float)S.nz * S.dz;
    w.inside = abs_vox(S, x[0], x[1], x[2], w.v[0], w.v[1], w.v[2]);
    if (!w.inside) { w.v[0] = w.v[1] = w.v[2] = 0; }
    w.r = r;
    w.s = s0;
    w.guard = 0;
    return w.s < w.r;
}

// one step of the walk; false once it has ended
__device__ __forceinline__ bool prange_walk_step(const SimDesc& S, PWalk& w)
{
    float step = 1000.0f;
    if (w.inside) {
        int ax = 0;
        const int px = w.pos & 1, py = (w.pos >> 1) & 1, pz = (w.pos >> 2) & 1;
        float bb = (S.offx + (float)(w.v[0] + px) * S.dx - w.x[0]) * w.id[0];
        if (step > bb) { step = bb; ax = 1; }
        bb = (S.offy + (float)(w.v[1] + py) * S.dy - w.x[1]) * w.id[1];
        if (step > bb) { step = bb; ax = 2; }
        bb = (S.offz + (float)(w.v[2] + pz) * S.dz - w.x[2]) * w.id[2];
        if (step > bb) { step = bb; ax = 3; }
        if (ax == 1) w.v[0] += px ? 1 : -1;
        else if (ax == 2) w.v[1] += py ? 1 : -1;
        else w.v[2] += pz ? 1 : -1;
        float rho = den_clamped(S, w.v[0], w.v[1], w.v[2]);
        step = step * w.r;
        w.s += step * rho;
        if (w.s > w.r) step += (w.r - w.s) / rho;
    } else {
        step = (w.r - w.s) / 0.0012905f;
        w.s = w.r + 100.0f;
    }
    w.x[0] += step * w.dn[0];
    w.x[1] += step * w.dn[1];
    w.x[2] += step * w.dn[2];
    if (w.x[0] < S.offx || w.x[0] > w.xmax) w.inside = false;
    if (w.x[1] < S.offy || w.x[1] > w.ymax) w.inside = false;
    if (w.x[2] < S.offz || w.x[2] > w.zmax) w.inside = false;
    ++w.guard;
    return w.s < w.r && w.guard < 100000;
}

// ---------------------------------------------------------------- photons
// t is the emission time stamp (double, us); tf the flight time since then in
// single precision, added to t once when the photon leaves the stage (FP64
// arithmetic on GB300 is ~64x slower than FP32; one double add per photon
// instead of a double division per step)
struct Photon {
    float x[3], u[3], E;
    double t;
    float tf;
    int nscat;
};

// annihilation pair, setPosition gPET_kernals.cu:536-555 (non-collinearity
// with the +-theta*MC2/2 energy shift of the reference)
// spare: a standard normal already drawn (the positron range's second
// normal of its last pair) for the non-collinearity angle, or null
__device__ __forceinline__ void make_pair(const SimDesc& S, Stream& st, const float pos[3], double t_us, Photon ph[2],
                                          const float* spare = nullptr)
{
    float cost = -1.0f + 2.0f * st_u(st);
    float phi = st_u(st);
    float s, c;
    dm_sincos_turns(phi, &s, &c);
    float sint = dm_sqrt(1.0f - cost * cost);
    float u0 = sint * c, u1 = sint * s, u2 = cost;
    float phi2 = st_u(st);
    float theta = (spare ? *spare : st_normal(st)) * S.noncol_sigma;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        ph[k].x[0] = pos[0]; ph[k].x[1] = pos[1]; ph[k].x[2] = pos[2];
        ph[k].t = t_us; ph[k].tf = 0.0f; ph[k].nscat = 0;
    }
    ph[0].u[0] = u0; ph[0].u[1] = u1; ph[0].u[2] = u2;
    ph[0].E = kMC2 + theta * kMC2 / 2.0f;
    float ts, tc;
    dm_sincos_turns(theta * 0.159154943091895335768883763f, &ts, &tc);
    rotate(u0, u1, u2, -tc, phi2);
    ph[1].u[0] = u0; ph[1].u[1] = u1; ph[1].u[2] = u2;
    ph[1].E = kMC2 - theta * kMC2 / 2.0f;
}

// comsam(matid), gPET_kernals.cu:66-88
template <class U>
__device__ __forceinline__ void compton_surface_u(const SimDesc& S, float e, int m, U&& unif, float& efrac,
                                                  float& cost)
{
    float indcp = unif() * S.idcp_c;
    float inde = e * S.ide_c;
    float c = lerp2(S.cmpsf + (size_t)m * S.ncp_c * S.ne_c, S.ncp_c, S.ne_c, inde, indcp);
    if (c > 1.0f) c = 1.0f;
    if (c < -1.0f) c = -1.0f;
    cost = c;
    efrac = 1.0f / (1.0f + e * kIMC2 * (1.0f - c));
}

__device__ __forceinline__ void compton_surface(const SimDesc& S, float e, int m, Stream& st, float& efrac, float& cost)
{
    compton_surface_u(S, e, m, [&]() { return st_u(st); }, efrac, cost);
}

// rylsam, gPET_kernals.cu:128-146
template <class U>
__device__ __forceinline__ float rayleigh_surface_u(const SimDesc& S, float e, int m, U&& unif)
{
    float indcp = unif() * S.idcp_r;
    float inde = e * S.ide_r;
    float c = lerp2(S.rayff + (size_t)m * S.ncp_r * S.ne_r, S.ncp_r, S.ne_r, inde, indcp);
    if (c > 1.0f) c = 1.0f;
    if (c < -1.0f) c = -1.0f;
    return c;
}

__device__ __forceinline__ float rayleigh_surface(const SimDesc& S, float e, int m, Stream& st)
{
    return rayleigh_surface_u(S, e, m, [&]() { return st_u(st); });
}

// comsam, free-electron Klein-Nishina, gPET_kernals.cu:90-126
template <class U>
__device__ __forceinline__ void kn_sample_u(float e, U&& unif, float& efrac, float& cost)
{
    float e0 = e * kIMC2;
    float twoe = 2.0f * e0;
    float kmin2 = 1.0f / ((1.0f + twoe) * (1.0f + twoe));
    float loge = dm_logf(1.0f + twoe);
    float ef = 1.0f;
    for (int it = 0; it < 100000; ++it) {
        if (unif() * (loge + twoe * (1.0f + e0) * kmin2) < loge)
            ef = dm_expf(-unif() * loge);
        else
            ef = dm_sqrt(kmin2 + unif() * (1.0f - kmin2));
        float mess = e0 * e0 * ef * (1.0f + ef * ef);
        if (unif() * mess <= mess - (1.0f - ef) * ((1.0f + twoe) * ef - 1.0f)) break;
    }
    efrac = ef;
    cost = 1.0f - (1.0f - ef) / (ef * e0);
}

__device__ __forceinline__ void kn_sample(float e, Stream& st, float& efrac, float& cost)
{
    kn_sample_u(e, [&]() { return st_u(st); }, efrac, cost);
}

// photon(), gPET_kernals.cu:256-345 - Woodcock tracking to the phantom exit.
// Returns 0 photoelectric, 1 escaped (or fell below eabsph after a Compton
// event and leaves as-is, :318-320), 3 step cap. `steps` counts iterations.
__device__ __forceinline__ int phantom_transport(const SimDesc& S, Photon& p, Stream& st, int& steps)
{
    for (int step = 0; step < kMaxSteps; ++step) {
        steps++;
        float lammin = wck_at(S.wck_ph, S.wck_e0, S.wck_ide, p.E);
        float s = -lammin * dm_logf(st_u(st));
        p.x[0] = dm_fma(s, p.u[0], p.x[0]);
        p.x[1] = dm_fma(s, p.u[1], p.x[1]);
        p.x[2] = dm_fma(s, p.u[2], p.x[2]);
        p.tf = dm_fma(s, DM_INV_SPEED, p.tf);
        int ix, iy, iz;
        if (!abs_vox(S, p.x[0], p.x[1], p.x[2], ix, iy, iz)) return 1;
        uint2 vv = voxel(S, ix, iy, iz);
        float voxden = __uint_as_float(vv.x);
        int m = (int)vv.y;
        float lamden = lammin * voxden;
        float4 xs = xs_at(S, m, p.E);
        float prob = dm_fma(-lamden, xs.x, 1.0f);
        float rn = st_u(st);
        if (rn < prob) continue;
        prob = dm_fma(lamden, xs.y, prob);
        if (rn < prob) {
            float efrac, cost;
            compton_surface(S, p.E, m, st, efrac, cost);
            float phi = st_u(st);
            p.E *= efrac;
            p.nscat++;
            if (p.E < S.eabsph) return 1;
            rotate(p.u[0], p.u[1], p.u[2], cost, phi);
            continue;
        }
        prob = dm_fma(lamden, xs.z, prob);
        if (rn < prob) {
            float cost = rayleigh_surface(S, p.E, m, st);
            float phi = st_u(st);
            rotate(p.u[0], p.u[1], p.u[2], cost, phi);
            p.nscat++;
            continue;
        }
        return 0;
    }
    return 3;
}

// entry state in a panel's local frame: t the entry time stamp, tf the
// flight time inside the panel since then
struct Local {
    float x[3], u[3], E;
    double t;
    float tf;
    int panel;
};

// panel search of photonde, gPET_kernals.cu:963-1009 (panels staged in
// shared memory)
// False only when the photon's line cannot meet any panel entry face: while
// it is inside the faces' z range it stays closer to the z axis than every
// face (its squared distance to the axis is convex along the line, so the
// two ends of that range bound it). enter_panel would then find nothing; the
// bounds are padded, so this never changes a result.
__device__ __forceinline__ bool may_reach_panels(const SimDesc& S, const Photon& p)
{
    if (!S.ring_test) return true;
    const float uz = p.u[2];
    if (uz == 0.0f) return p.x[2] >= S.ring_zmin && p.x[2] <= S.ring_zmax;
    const float iu = 1.0f / uz;
    const float t1 = (S.ring_zmin - p.x[2]) * iu, t2 = (S.ring_zmax - p.x[2]) * iu;
    const float tb = fmaxf(t1, t2);
    float ta = fminf(t1, t2);
    // ring_test 2: every face takes only photons moving toward it from the
    // axis side, so for a photon inside the faces' cylinder only the part of
    // the ray ahead of it counts (a photon leaving the z band never reaches a
    // face)
    if (S.ring_test == 2 && p.x[0] * p.x[0] + p.x[1] * p.x[1] < S.ring_rin2) {
        if (tb < 0.0f) return false;
        ta = fmaxf(ta, 0.0f);
    }
    const float x1 = p.x[0] + ta * p.u[0], y1 = p.x[1] + ta * p.u[1];
    const float x2 = p.x[0] + tb * p.u[0], y2 = p.x[1] + tb * p.u[1];
    return fmaxf(x1 * x1 + y1 * y1, x2 * x2 + y2 * y2) >= S.ring_rin2;
}

__device__ __forceinline__ bool enter_panel(const float* __restrict__ P0, int npanels, const Photon& p, Local& q)
{
    for (int i = 0; i < npanels; ++i) {
        const float* P = P0 + i * kPanelStride;
        // the direction test first: the other projections are only needed
        // for a panel the photon moves toward (values are unchanged)
        float tvx = p.u[0] * P[21] + p.u[1] * P[22] + p.u[2] * P[23];
        if (!(tvx * P[18] >= 0.0f)) continue;
        float px = p.x[0] - P[15], py = p.x[1] - P[16], pz = p.x[2] - P[17];
        float tx = px * P[21] + py * P[22] + pz * P[23];
        float ty = px * P[24] + py * P[25] + pz * P[26];
        float tz = px * P[27] + py * P[28] + pz * P[29];
        float tvy = p.u[0] * P[24] + p.u[1] * P[25] + p.u[2] * P[26];
        float tvz = p.u[0] * P[27] + p.u[1] * P[28] + p.u[2] * P[29];
        {
            float ty2 = ty - tx / tvx * tvy;
            float tz2 = tz - tx / tvx * tvz;
            if (fabsf(ty2) < P[1] / 2.0f && fabsf(tz2) < P[2] / 2.0f) {
                q.x[0] = 0.0f; q.x[1] = ty2; q.x[2] = tz2;
                q.u[0] = tvx; q.u[1] = tvy; q.u[2] = tvz;
                q.E = p.E;
                q.t = p.t + (double)(p.tf + -tx / tvx * DM_INV_SPEED);
                q.tf = 0.0f;
                q.panel = i;
                return true;
            }
        }
    }
    return false;
}

// crystalSearch, gPET_kernals.cu:1236-1279 (m_id 0 crystal, 1 gap). A point
// inside quadratic surface k is gap (the reference), or, when the detector
// lists a material 2 + k, crystal of that material (still gap between
// crystals)
__device__ __forceinline__ void crystal_search(const SimDesc& S, const float* P, const float x[3], int& m_id,
                                               int& M_id, int& L_id)
{
    float xx = x[0], y = x[1], z = x[2];
    int region = 0;
    for (int k = 0; k < S.nsurface; ++k) {
        const float* a = S.surface + 10 * k;
        float v = a[0] * xx * xx + a[1] * y * y + a[2] * z * z + a[3] * xx * y + a[4] * xx * z + a[5] * y * z +
                  a[6] * xx + a[7] * y + a[8] * z + a[9];
        if (v < 0.0f) {
            if (2 + k < S.ndetmat) { region = 2 + k; break; }
            m_id = 1;
            return;
        }
    }
    y = P[1] / 2.0f + x[1];
    z = P[2] / 2.0f + x[2];
    float pmy = P[4] + P[7], pmz = P[5] + P[8];
    int my = floorf(y / pmy) > 0.0f ? (int)(y / pmy) : 0;
    int mz = floorf(z / pmz) > 0.0f ? (int)(z / pmz) : 0;
    M_id = mz * S.moduleNy + my;
    y = y - (float)my * pmy;
    z = z - (float)mz * pmz;
    if (y > P[4] || z > P[5]) { m_id = 1; return; }
    float pcy = P[10] + P[13], pcz = P[11] + P[14];
    int ly = floorf(y / pcy) > 0.0f ? (int)(y / pcy) : 0;
    int lz = floorf(z / pcz) > 0.0f ? (int)(z / pcz) : 0;
    L_id = lz * S.crystalNy + ly;
    y = y - (float)ly * pcy;
    z = z - (float)lz * pcz;
    if (y > P[10] || z > P[11]) { m_id = 1; return; }
    m_id = region;
}

}  // namespace gpet
