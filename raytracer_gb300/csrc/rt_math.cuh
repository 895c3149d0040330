// rt_math.cuh -- scalar/vector arithmetic and the PCG32 stream on the device.
//
// Every routine reproduces the reference renderer's evaluation order in IEEE
// binary32 (the library is compiled with -fmad=false, so a*b+c stays two
// rounded operations, as on the reference's CPU build).  Vector redux order
// follows Eigen's 3-vector dot: (a0*b0 + a1*b1) + a2*b2.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#define RT_PI 3.14159265358979323846f
#define RT_INV_PI 0.3183098861837906715377f
#define RT_INV_FOUR_PI 0.07957747154594766788450883936693f
#define RT_MAX_REAL 10e7f
#define RT_EPSILON 1e-4f

struct V3 { float x, y, z; };
struct C3 { float r, g, b; };
struct V2 { float x, y; };

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
__host__ __device__ __forceinline__ C3 c3(float r, float g, float b) { C3 c; c.r = r; c.g = g; c.b = b; return c; }
__host__ __device__ __forceinline__ C3 cfill(float v) { return c3(v, v, v); }

// std::min / std::max semantics (first argument returned on ties / NaN)
__host__ __device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ int imin(int a, int b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ int imax(int a, int b) { return (a < b) ? b : a; }

__host__ __device__ __forceinline__ float vget(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float sqnorm(V3 a) { return dot(a, a); }
__host__ __device__ __forceinline__ float norm(V3 a) { return sqrtf(sqnorm(a)); }
// Eigen normalized(): v / sqrt(squaredNorm) when non-zero, else v
__host__ __device__ __forceinline__ V3 normalized(V3 a)
{
    float n = sqnorm(a);
    if (n > 0.f) return a / sqrtf(n);
    return a;
}

__host__ __device__ __forceinline__ C3 operator+(C3 a, C3 b) { return c3(a.r + b.r, a.g + b.g, a.b + b.b); }
__host__ __device__ __forceinline__ C3 operator*(C3 a, C3 b) { return c3(a.r * b.r, a.g * b.g, a.b * b.b); }
__host__ __device__ __forceinline__ C3 operator*(C3 a, float s) { return c3(a.r * s, a.g * s, a.b * s); }
__host__ __device__ __forceinline__ C3 operator*(float s, C3 a) { return c3(s * a.r, s * a.g, s * a.b); }
__host__ __device__ __forceinline__ C3 operator/(C3 a, float s) { return c3(a.r / s, a.g / s, a.b / s); }
__host__ __device__ __forceinline__ C3 operator/(C3 a, C3 b) { return c3(a.r / b.r, a.g / b.g, a.b / b.b); }
// core/Color.h:151-158 average(): running sum from 0, then / 3
__host__ __device__ __forceinline__ float cavg(C3 a) { float s = 0.f; s += a.r; s += a.g; s += a.b; return s / 3.f; }
__host__ __device__ __forceinline__ float cavg1(float v) { float s = 0.f; s += v; s += v; s += v; return s / 3.f; }
// core/Color.h:423-426
__host__ __device__ __forceinline__ float lum(C3 a) { return 0.2126f * a.r + 0.7152f * a.g + 0.0722f * a.b; }
// core/Color.h:163-171 isZero(1e-5)
__host__ __device__ __forceinline__ bool iszero(C3 a)
{
    return fabsf(a.r) <= 1e-5f && fabsf(a.g) <= 1e-5f && fabsf(a.b) <= 1e-5f;
}
__host__ __device__ __forceinline__ bool cisnan(C3 a) { return isnan(a.r) || isnan(a.g) || isnan(a.b); }
__host__ __device__ __forceinline__ float cmax(C3 a) { return smax(a.r, smax(a.g, a.b)); }
__host__ __device__ __forceinline__ C3 cload(const float *p) { return c3(p[0], p[1], p[2]); }
__host__ __device__ __forceinline__ V3 vload(const float *p) { return v3(p[0], p[1], p[2]); }

// core/Transform.h:90-99 (point), :118-125 (vector), :181-189 (normal)
__host__ __device__ __forceinline__ V3 xf_point(const float *m, V3 p)
{
    V3 o;
    o.x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    o.y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    o.z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    float w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    if (w != 1.f && w != 0.f) o = o / w;
    return o;
}
__host__ __device__ __forceinline__ V3 xf_vector(const float *m, V3 v)
{
    return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z,
              m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
__host__ __device__ __forceinline__ V3 xf_normal(const float *inv, V3 n)
{
    return v3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z,
              inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
              inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

// ---------------------------------------------------------------- PCG32
// tools/Rng.h:81-141 (seed, XSH-RR output, mantissa float)
#define RT_PCG_MULT 0x5851f42d4c957f2dULL

struct Pcg32 { uint64_t state, inc; };

__host__ __device__ __forceinline__ uint32_t pcg_next(Pcg32 &r)
{
    uint64_t old = r.state;
    r.state = old * RT_PCG_MULT + r.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((~rot + 1u) & 31));
}
__host__ __device__ __forceinline__ void pcg_seed(Pcg32 &r, uint64_t initstate, uint64_t initseq)
{
    r.state = 0u;
    r.inc = (initseq << 1u) | 1u;
    pcg_next(r);
    r.state += initstate;
    pcg_next(r);
}
__host__ __device__ __forceinline__ float pcg_float(Pcg32 &r)
{
    uint32_t u = (pcg_next(r) >> 9) | 0x3f800000u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(u) - 1.0f;
#else
    union { uint32_t u; float f; } x;
    x.u = u;
    return x.f - 1.0f;
#endif
}
// splitmix64 finaliser: per-path initial state of the path-stream sampler
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}
__host__ __device__ __forceinline__ void path_stream_seed(Pcg32 &r, uint64_t seed, uint32_t pixel, uint32_t sample)
{
    pcg_seed(r, mix64((seed << 32) ^ (uint64_t)pixel), (uint64_t)sample);
}
__host__ __device__ __forceinline__ float next1d(Pcg32 &r) { return pcg_float(r); }
__host__ __device__ __forceinline__ V2 next2d(Pcg32 &r)
{
    float a = pcg_float(r);
    float b = pcg_float(r);
    return v2(a, b);
}
