/*
 * OpenCL C 1.2 shim: just enough of the OpenCL C language and built-ins for
 * the reference's kernel files to compile unmodified as C++ and run on the
 * host, one NDRange at a time (ref_kernels.cpp).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * The image sampler follows the OpenCL 1.2 specification, section 8
 * (unnormalised coordinates; CLK_FILTER_NEAREST: i = floor(u);
 * CLK_FILTER_LINEAR: i0 = floor(u - 0.5), a = frac(u - 0.5),
 * T = (1-a)(1-b)T00 + a(1-b)T10 + (1-a)bT01 + abT11; CLK_ADDRESS_CLAMP
 * returns the border colour outside the image, CLK_ADDRESS_CLAMP_TO_EDGE
 * clamps the index). Images are single-channel float (CL_R): a texel reads
 * as (v, 0, 0, 1), the border colour is (0, 0, 0, 1).
 *
 * The sampler's arithmetic order inside a real OpenCL runtime is not part of
 * the reference; this shim and the C restatement in oracle_impl.inc use the
 * same spec formula, so they agree bit for bit.
 */
#ifndef UFOIR_CLSHIM_HPP
#define UFOIR_CLSHIM_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <sys/types.h>

using std::ceil;
using std::fabs;
using std::floor;
using std::pow;
using std::sqrt;

namespace clshim {
extern thread_local size_t gid[3];
extern thread_local size_t gsize[3];
}

typedef unsigned int uint;
typedef int sampler_t;

enum {
    CLK_NORMALIZED_COORDS_FALSE = 0,
    CLK_NORMALIZED_COORDS_TRUE = 1,
    CLK_ADDRESS_NONE = 0,
    CLK_ADDRESS_CLAMP_TO_EDGE = 2,
    CLK_ADDRESS_CLAMP = 4,
    CLK_ADDRESS_REPEAT = 8,
    CLK_FILTER_NEAREST = 16,
    CLK_FILTER_LINEAR = 32,
};

struct float2 {
    float x, y;
};

/* Members are mutable and the default constructor is user-provided so that
 * the reference's "const int2 c; c.x = ...;" (projector-parallel-joseph.cl:169-171)
 * compiles as written. */
struct int2 {
    mutable int x, y;
    int2() {}
};

struct float4 {
    union { float x; float s0; };
    union { float y; float s1; };
    union { float z; float s2; };
    union { float w; float s3; };
    float4() {}
    float4(float v) { x = v; y = v; z = v; w = v; }
    float4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
};

static inline float4 operator+(const float4 &a, const float4 &b)
{
    return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
static inline float4 &operator+=(float4 &a, const float4 &b)
{
    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
    return a;
}
static inline float4 operator*(const float4 &a, float s)
{
    return float4(a.x * s, a.y * s, a.z * s, a.w * s);
}
static inline float4 operator*(float s, const float4 &a)
{
    return float4(s * a.x, s * a.y, s * a.z, s * a.w);
}

struct image2d_t {
    float *data;
    long width;
    long height;
};

template <typename T> static inline float convert_float(T v) { return (float) v; }

static inline size_t get_global_id(uint d) { return clshim::gid[d]; }
static inline size_t get_global_size(uint d) { return clshim::gsize[d]; }

static inline float4 clshim_texel(const image2d_t &img, long i, long j, sampler_t s)
{
    if (s & CLK_ADDRESS_CLAMP_TO_EDGE) {
        if (i < 0) i = 0;
        if (j < 0) j = 0;
        if (i >= img.width) i = img.width - 1;
        if (j >= img.height) j = img.height - 1;
    } else if (i < 0 || j < 0 || i >= img.width || j >= img.height) {
        return float4(0.0f, 0.0f, 0.0f, 1.0f);
    }
    return float4(img.data[(size_t) j * (size_t) img.width + (size_t) i], 0.0f, 0.0f, 1.0f);
}

static inline float4 read_imagef(image2d_t img, sampler_t s, float2 c)
{
    if (s & CLK_FILTER_LINEAR) {
        const float um = c.x - 0.5f;
        const float vm = c.y - 0.5f;
        const float fi = std::floor(um);
        const float fj = std::floor(vm);
        const long i0 = (long) fi, j0 = (long) fj;
        const float a = um - fi;
        const float b = vm - fj;
        const float4 t00 = clshim_texel(img, i0, j0, s);
        const float4 t10 = clshim_texel(img, i0 + 1, j0, s);
        const float4 t01 = clshim_texel(img, i0, j0 + 1, s);
        const float4 t11 = clshim_texel(img, i0 + 1, j0 + 1, s);
        float4 r;
        r.x = (1 - a) * (1 - b) * t00.x + a * (1 - b) * t10.x + (1 - a) * b * t01.x + a * b * t11.x;
        r.y = (1 - a) * (1 - b) * t00.y + a * (1 - b) * t10.y + (1 - a) * b * t01.y + a * b * t11.y;
        r.z = (1 - a) * (1 - b) * t00.z + a * (1 - b) * t10.z + (1 - a) * b * t01.z + a * b * t11.z;
        r.w = (1 - a) * (1 - b) * t00.w + a * (1 - b) * t10.w + (1 - a) * b * t01.w + a * b * t11.w;
        return r;
    }
    return clshim_texel(img, (long) std::floor(c.x), (long) std::floor(c.y), s);
}

static inline float4 read_imagef(image2d_t img, sampler_t s, int2 c)
{
    return clshim_texel(img, c.x, c.y, s);
}

static inline void write_imagef(image2d_t img, int2 c, float4 v)
{
    if (c.x < 0 || c.y < 0 || c.x >= img.width || c.y >= img.height)
        return;
    img.data[(size_t) c.y * (size_t) img.width + (size_t) c.x] = v.x;
}

/* OpenCL C address-space and access qualifiers carry no meaning here. */
#define kernel
#define __kernel
#define global
#define __global
#define constant const
#define __constant const
#define read_only
#define write_only
#define __read_only
#define __write_only

#endif
