// cl_shim.hpp -- a minimal OpenCL-C environment for compiling the reference's OpenCL 1.2
// kernel sources as C++ on the host (TEST INFRASTRUCTURE ONLY: it builds oracle/_ref, the
// checker that pins the oracle; nothing in the product uses it).
//
// The kernel sources are included inside namespace clk, so the builtins below shadow the
// C library's.  The image/sampler behaviour follows the OpenCL 1.2 specification
// (section 8, "Image Addressing and Filtering"): unnormalised coordinates,
// CLK_ADDRESS_CLAMP with the CL_R border colour (.x == 0), linear filtering with
// i0 = floor(u - 0.5) and a = frac(u - 0.5), nearest filtering with i = floor(u), array
// layer = clamp(rint(z)), CLK_ADDRESS_CLAMP_TO_EDGE clamping texel indices to the edge.
// cos/sin of a float are taken correctly rounded
// ((float)cos((double)x)); the specification allows up to 4 ulp.
#pragma once
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#define __kernel
#define kernel
#define __read_only
#define __write_only
#define __read_write
#define __global
#define __local
#define __private
#define __constant const

namespace clk {

// ---- vector types (only what the kernels use: construction, .x/.y/.z/.w, the float2
// arithmetic and swizzles of FBP.cl, as_float2/as_uint2 bit casts) ----
struct float4 {
    float x, y, z, w;
    float4() : x(0), y(0), z(0), w(0) {}
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};
struct int4 {
    int x, y, z, w;
    int4() : x(0), y(0), z(0), w(0) {}
    int4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
};
struct float2 {
    float x, y;
    float2() : x(0), y(0) {}
    float2(float a, float b) : x(a), y(b) {}
    // swizzles: the build rewrites v.xx / v.yy / v.yx into these calls
    float2 xx() const { return float2(x, x); }
    float2 yy() const { return float2(y, y); }
    float2 yx() const { return float2(y, x); }
    float2 &operator*=(float s) { x *= s; y *= s; return *this; }
    float2 &operator/=(float s) { x /= s; y /= s; return *this; }
    float2 &operator+=(float2 o) { x += o.x; y += o.y; return *this; }
};
inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator*(float2 a, float2 b) { return float2(a.x * b.x, a.y * b.y); }
inline float2 operator*(float s, float2 b) { return float2(s * b.x, s * b.y); }
inline float2 &operator-=(float2 &a, float2 b)
{
    a = float2(a.x - b.x, a.y - b.y);
    return a;
}
typedef unsigned int uint;
struct uint2 {
    uint x, y;
    uint2() : x(0), y(0) {}
    uint2(uint a, uint b) : x(a), y(b) {}
};
inline uint2 operator^(uint2 a, uint2 b) { return uint2(a.x ^ b.x, a.y ^ b.y); }
inline uint2 as_uint2(float2 v)
{
    uint2 r;
    memcpy(&r.x, &v.x, 4);
    memcpy(&r.y, &v.y, 4);
    return r;
}
inline float2 as_float2(uint2 v)
{
    float2 r;
    memcpy(&r.x, &v.x, 4);
    memcpy(&r.y, &v.y, 4);
    return r;
}
struct int2 {
    int x, y;
    int2() : x(0), y(0) {}
    int2(int a, int b) : x(a), y(b) {}
};

// ---- samplers ----
typedef int sampler_t;
enum {
    CLK_NORMALIZED_COORDS_FALSE = 0,
    CLK_NORMALIZED_COORDS_TRUE = 1,
    CLK_ADDRESS_NONE = 0,
    CLK_ADDRESS_CLAMP = 2,
    CLK_ADDRESS_CLAMP_TO_EDGE = 4,
    CLK_FILTER_NEAREST = 0,
    CLK_FILTER_LINEAR = 16,
};
enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };

// ---- images: one float (CL_R, CL_FLOAT) per texel, layers stacked ----
struct image2d_array_t {
    float *data;
    int w, h, d;
};
struct image2d_t {
    float *data;
    int w, h;
};

// Undefined case of the reference (read_imagef with a LINEAR sampler at int coords):
// 0 = exact texel, 1 = treat the coords as float and filter.
extern int g_int_linear_mode;

inline float texel_(const image2d_array_t &im, int i, int j, int k)
{
    if (i < 0 || j < 0 || i >= im.w || j >= im.h) return 0.0f;  // CLK_ADDRESS_CLAMP border
    return im.data[((size_t)k * im.h + j) * im.w + i];
}
// CLK_ADDRESS_CLAMP_TO_EDGE: out-of-range texels take the nearest edge texel
inline float texel_edge_(const image2d_array_t &im, int i, int j, int k)
{
    i = i < 0 ? 0 : (i >= im.w ? im.w - 1 : i);
    j = j < 0 ? 0 : (j >= im.h ? im.h - 1 : j);
    return im.data[((size_t)k * im.h + j) * im.w + i];
}
inline float texel_mode_(const image2d_array_t &im, int smp, int i, int j, int k)
{
    return (smp & CLK_ADDRESS_CLAMP_TO_EDGE) ? texel_edge_(im, i, j, k) : texel_(im, i, j, k);
}
inline int layer_(const image2d_array_t &im, float z)
{
    int k = (int)rintf(z);
    return k < 0 ? 0 : (k >= im.d ? im.d - 1 : k);
}
inline float4 read_imagef(image2d_array_t im, sampler_t smp, float4 c)
{
    const int k = layer_(im, c.z);
    if (smp & CLK_FILTER_LINEAR) {
        const float u = c.x - 0.5f, v = c.y - 0.5f;
        const float fi = floorf(u), fj = floorf(v);
        const float a = u - fi, b = v - fj;
        const int i = (int)fi, j = (int)fj;
        const float t = (1.0f - a) * (1.0f - b) * texel_mode_(im, smp, i, j, k) +
                        a * (1.0f - b) * texel_mode_(im, smp, i + 1, j, k) +
                        (1.0f - a) * b * texel_mode_(im, smp, i, j + 1, k) + a * b * texel_mode_(im, smp, i + 1, j + 1, k);
        return float4(t, 0.0f, 0.0f, 1.0f);
    }
    return float4(texel_mode_(im, smp, (int)floorf(c.x), (int)floorf(c.y), k), 0.0f, 0.0f, 1.0f);
}
inline float4 read_imagef(image2d_array_t im, sampler_t smp, int4 c)
{
    if ((smp & CLK_FILTER_LINEAR) && g_int_linear_mode == 1)
        return read_imagef(im, smp, float4((float)c.x, (float)c.y, (float)c.z, 0.0f));
    const int k = c.z < 0 ? 0 : (c.z >= im.d ? im.d - 1 : c.z);
    return float4(texel_(im, c.x, c.y, k), 0.0f, 0.0f, 1.0f);
}
inline void write_imagef(image2d_array_t im, int4 c, float4 v)
{
    if (c.x < 0 || c.y < 0 || c.z < 0 || c.x >= im.w || c.y >= im.h || c.z >= im.d) return;
    im.data[((size_t)c.z * im.h + c.y) * im.w + c.x] = v.x;
}
inline float4 read_imagef(image2d_t im, sampler_t smp, float2 c)
{
    image2d_array_t a = {im.data, im.w, im.h, 1};
    return read_imagef(a, smp, float4(c.x, c.y, 0.0f, 0.0f));
}
inline void write_imagef(image2d_t im, int2 c, float4 v)
{
    image2d_array_t a = {im.data, im.w, im.h, 1};
    write_imagef(a, int4(c.x, c.y, 0, 0), v);
}

// ---- work-item functions: the driver sets these per work-item ----
extern thread_local size_t g_gid[3];
extern thread_local size_t g_lid[3];
extern thread_local size_t g_lsz[3];
extern thread_local size_t g_grp[3];
// Drivers that run a work-group as one host thread per work-item install a real barrier
// here; kernels driven one work-item at a time have none and need none.
extern thread_local void (*g_barrier_fn)(void);
inline size_t get_global_id(int d) { return g_gid[d]; }
inline size_t get_local_id(int d) { return g_lid[d]; }
inline size_t get_local_size(int d) { return g_lsz[d]; }
inline size_t get_group_id(int d) { return g_grp[d]; }
extern thread_local size_t g_gsz[3];   // global size (set by drivers whose kernels ask)
inline size_t get_global_size(int d) { return g_gsz[d]; }
inline size_t get_num_groups(int d) { return g_gsz[d] / (g_lsz[d] ? g_lsz[d] : 1); }
inline void barrier(int)
{
    if (g_barrier_fn) g_barrier_fn();
}

// ---- math builtins (float overloads as in OpenCL C) ----
inline float cos(float x) { return (float)::cos((double)x); }
inline float sin(float x) { return (float)::sin((double)x); }
inline double cos(double x) { return ::cos(x); }
inline double sin(double x) { return ::sin(x); }
inline float2 cos(float2 v) { return float2(cos(v.x), cos(v.y)); }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float asin(float x) { return (float)::asin((double)x); }
inline float exp(float x) { return (float)::exp((double)x); }
inline float sqrt(float x) { return ::sqrtf(x); }
inline float fabs(float x) { return ::fabsf(x); }
inline float fmin(float a, float b) { return ::fminf(a, b); }
inline float fmax(float a, float b) { return ::fmaxf(a, b); }
inline float max(float a, float b) { return (a < b) ? b : a; }
inline float min(float a, float b) { return (b < a) ? b : a; }
inline int max(int a, int b) { return (a < b) ? b : a; }
inline int min(int a, int b) { return (b < a) ? b : a; }
inline int isnan(float x) { return x != x; }

}  // namespace clk
