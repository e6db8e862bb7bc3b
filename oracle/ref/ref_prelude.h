/* ref_prelude.h - CPU stand-ins for the CUDA runtime, texture, curand and
 * vector-type names used by the reference's own source, so that selected
 * reference functions compile with g++ and run on the host (TEST
 * INFRASTRUCTURE: only the pins in tests/ use the library built from them).
 *
 * What each stand-in does:
 *  - __device__/__global__/__host__/__constant__: nothing (host code);
 *    __shared__ becomes `static` (one serial "thread" per call).
 *  - threadIdx/blockIdx = 0, blockDim/gridDim = 1: a kernel body runs as one
 *    thread; the harness calls it once per photon.
 *  - texture<T, dim, mode>: unnormalised coordinates, clamp addressing, point
 *    or linear filtering as the reference sets it (filterMode). Linear
 *    filtering takes the full FP32 fraction (the oracle's convention);
 *    ref_tex_frac_bits > 0 rounds the fraction to that many bits instead, as
 *    texture hardware does.
 *  - curand: curand_uniform returns the next word of a tape through
 *    dm_u01, the oracle's own conversion, so both sides see the same
 *    uniforms; curand_normal is Box-Muller (dm_normal2) on two uniforms with
 *    the second normal cached in the state for the next call.
 *  - cudaMalloc*, cudaMemcpy*, cudaMemcpyToSymbol, cudaBindTexture*: host
 *    memory and plain copies.
 *  - __logf/__expf/__sinf/__cosf/__fsqrt_rn: the libm functions.
 */
#ifndef REF_PRELUDE_H
#define REF_PRELUDE_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <vector>
#include <unistd.h>

#include "detmath.h"

using std::abs;   /* abs() of a float is the float overload, as in device code */

#define __device__
#define __global__
#define __host__
#define __constant__
#define __shared__ static
#define __forceinline__ inline

/* ---------------------------------------------------------------- vectors */
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct int4 { int x, y, z, w; };
struct uint3 { unsigned x, y, z; };
struct dim3 { unsigned x, y, z; };
static inline float3 make_float3(float x, float y, float z) { return float3{x, y, z}; }
static inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
static inline int4 make_int4(int x, int y, int z, int w) { return int4{x, y, z, w}; }

static uint3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0};
static dim3 blockDim = {1, 1, 1}, gridDim = {1, 1, 1};
static inline void __syncthreads() {}

#define __logf(x) logf(x)
#define __expf(x) expf(x)
#define __sinf(x) sinf(x)
#define __cosf(x) cosf(x)
static inline float __fsqrt_rn(float x) { return sqrtf(x); }
static inline float __fdividef(float a, float b) { return a / b; }
template <class T> static inline T atomicAdd(T* p, T v) { T o = *p; *p = o + v; return o; }
template <class T> static inline T atomicSub(T* p, T v) { T o = *p; *p = o - v; return o; }

/* ----------------------------------------------------------- CUDA runtime */
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaTextureFilterMode { cudaFilterModePoint, cudaFilterModeLinear };
enum cudaTextureAddressMode { cudaAddressModeWrap, cudaAddressModeClamp, cudaAddressModeMirror, cudaAddressModeBorder };
enum cudaTextureReadMode { cudaReadModeElementType, cudaReadModeNormalizedFloat };
struct cudaChannelFormatDesc { int bytes; };
template <class T> static inline cudaChannelFormatDesc cudaCreateChannelDesc() { return cudaChannelFormatDesc{(int)sizeof(T)}; }
struct cudaExtent { size_t width, height, depth; };
static inline cudaExtent make_cudaExtent(size_t w, size_t h, size_t d) { return cudaExtent{w, h, d}; }
struct cudaPitchedPtr { void* ptr; size_t pitch, xsize, ysize; };
static inline cudaPitchedPtr make_cudaPitchedPtr(void* p, size_t pitch, size_t xs, size_t ys)
{
    return cudaPitchedPtr{p, pitch, xs, ys};
}
/* a "device array": w x h x d elements of 4 bytes (int or float) */
struct cudaArray {
    size_t w, h, d;
    std::vector<uint32_t> bits;
};
struct cudaMemcpy3DParms {
    cudaArray* srcArray; size_t srcPos[3]; cudaPitchedPtr srcPtr;
    cudaArray* dstArray; size_t dstPos[3]; cudaPitchedPtr dstPtr;
    cudaExtent extent; cudaMemcpyKind kind;
};
static inline cudaError_t cudaMallocArray(cudaArray** a, const cudaChannelFormatDesc*, size_t w, size_t h = 0)
{
    *a = new cudaArray{w, h ? h : 1, 1, std::vector<uint32_t>(w * (h ? h : 1))};
    return cudaSuccess;
}
static inline cudaError_t cudaMalloc3DArray(cudaArray** a, const cudaChannelFormatDesc*, cudaExtent e)
{
    *a = new cudaArray{e.width, e.height, e.depth, std::vector<uint32_t>(e.width * e.height * e.depth)};
    return cudaSuccess;
}
static inline cudaError_t cudaMemcpyToArray(cudaArray* a, size_t, size_t, const void* src, size_t bytes, cudaMemcpyKind)
{
    std::memcpy(a->bits.data(), src, bytes);
    return cudaSuccess;
}
static inline cudaError_t cudaMemcpy3D(const cudaMemcpy3DParms* p)
{
    std::memcpy(p->dstArray->bits.data(), p->srcPtr.ptr, p->extent.width * p->extent.height * p->extent.depth * 4);
    return cudaSuccess;
}
template <class T>
static inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t bytes, size_t off = 0,
                                             cudaMemcpyKind = cudaMemcpyHostToDevice)
{
    std::memcpy(reinterpret_cast<char*>(&sym) + off, src, bytes);
    return cudaSuccess;
}
template <class T>
static inline cudaError_t cudaMemcpyFromSymbol(void* dst, const T& sym, size_t bytes, size_t off = 0,
                                               cudaMemcpyKind = cudaMemcpyDeviceToHost)
{
    std::memcpy(dst, reinterpret_cast<const char*>(&sym) + off, bytes);
    return cudaSuccess;
}
static inline cudaError_t cudaMalloc(void** p, size_t n) { *p = std::calloc(1, n ? n : 1); return cudaSuccess; }
template <class T> static inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return cudaSuccess; }
static inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }

/* ---------------------------------------------------------------- textures */
extern int ref_tex_frac_bits;
template <class T, int dim, int mode = cudaReadModeElementType>
struct texture {
    int normalized = 0;
    cudaTextureFilterMode filterMode = cudaFilterModePoint;
    cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
    cudaChannelFormatDesc channelDesc = cudaCreateChannelDesc<T>();
    const cudaArray* arr = nullptr;
};
template <class T, int dim, int mode>
static inline cudaError_t cudaBindTextureToArray(texture<T, dim, mode>& t, const cudaArray* a)
{
    t.arr = a;
    return cudaSuccess;
}
template <class T, int dim, int mode>
static inline cudaError_t cudaBindTextureToArray(texture<T, dim, mode>& t, const cudaArray* a, const cudaChannelFormatDesc&)
{
    t.arr = a;
    return cudaSuccess;
}

template <class T> static inline T ref_texel(const cudaArray* a, long i, long j, long k)
{
    i = i < 0 ? 0 : (i >= (long)a->w ? (long)a->w - 1 : i);
    j = j < 0 ? 0 : (j >= (long)a->h ? (long)a->h - 1 : j);
    k = k < 0 ? 0 : (k >= (long)a->d ? (long)a->d - 1 : k);
    T v;
    std::memcpy(&v, &a->bits[(size_t)i + a->w * ((size_t)j + a->h * (size_t)k)], sizeof(T));
    return v;
}
/* texel index and weight of an unnormalised coordinate under linear filtering */
static inline void ref_tex_split(float x, long* i0, float* a)
{
    const float xb = x - 0.5f;
    const float f = floorf(xb);
    *i0 = (long)f;
    float w = xb - f;
    if (ref_tex_frac_bits > 0) {
        const float s = (float)(1 << ref_tex_frac_bits);
        w = rintf(w * s) / s;
    }
    *a = w;
}
template <class T, int mode> static inline T tex1D(const texture<T, 1, mode>& t, float x)
{
    if (t.filterMode == cudaFilterModePoint) return ref_texel<T>(t.arr, (long)floorf(x), 0, 0);
    long i; float a;
    ref_tex_split(x, &i, &a);
    const float v0 = (float)ref_texel<T>(t.arr, i, 0, 0), v1 = (float)ref_texel<T>(t.arr, i + 1, 0, 0);
    return (T)((1.0f - a) * v0 + a * v1);
}
template <class T, int mode> static inline T tex3D(const texture<T, 3, mode>& t, float x, float y, float z)
{
    if (t.filterMode == cudaFilterModePoint)
        return ref_texel<T>(t.arr, (long)floorf(x), (long)floorf(y), (long)floorf(z));
    long i, j, k; float a, b, c;
    ref_tex_split(x, &i, &a); ref_tex_split(y, &j, &b); ref_tex_split(z, &k, &c);
    float r = 0.0f;
    for (int dk = 0; dk < 2; ++dk)
        for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di) {
                const float w = (di ? a : 1.0f - a) * (dj ? b : 1.0f - b) * (dk ? c : 1.0f - c);
                r += w * (float)ref_texel<T>(t.arr, i + di, j + dj, k + dk);
            }
    return (T)r;
}

/* ------------------------------------------------------------------ curand */
struct curandState {
    const uint32_t* tape = nullptr;
    int64_t n = 0, pos = 0;
    int have_normal = 0;
    float normal = 0.0f;
};
static inline uint32_t ref_tape_word(curandState* s)
{
    const uint32_t w = s->pos < s->n ? s->tape[s->pos] : 0x80000000u;
    s->pos++;
    return w;
}
static inline float curand_uniform(curandState* s) { return dm_u01(ref_tape_word(s)); }
static inline double curand_uniform_double(curandState* s)
{
    const uint32_t hi = ref_tape_word(s), lo = ref_tape_word(s);
    return dm_u01d(hi, lo);
}
static inline float curand_normal(curandState* s)
{
    if (s->have_normal) {
        s->have_normal = 0;
        return s->normal;
    }
    const float u1 = curand_uniform(s), u2 = curand_uniform(s);
    float n1, n2;
    dm_normal2(u1, u2, &n1, &n2);
    s->have_normal = 1;
    s->normal = n2;
    return n1;
}
static inline void curand_init(unsigned long long, unsigned long long, unsigned long long, curandState* s) { *s = curandState(); }

#endif
