// clshim.hpp — TEST INFRASTRUCTURE.  Lets the reference's OpenCL C kernel
// sources (rtpslib/system/{common,sph}/cl_src/*.cl) compile as C++ and run on
// the host, so that the oracle can be pinned against the reference's own
// kernel code.  Nothing here is part of the product.
//
// What it supplies: the address-space qualifiers as no-ops, float4 / int4 with
// the .x/.y/.z/.w members and the .xyz swizzle the kernels use, component-wise
// vector arithmetic, the built-ins length / dot / max / get_*_id, and
// barrier() on top of a work-group emulator in which each work-item is a
// ucontext fiber (ref_runtime.cpp).  The build recipe (build_ref.py) rewrites
// the vector literal syntax `(float4)(a,b,c,d)` to `make_float4(a,b,c,d)`
// and turns kernel-scope `__local` arrays into statics; nothing else in the
// kernel sources changes.
//
// Semantics chosen where OpenCL leaves room (they match sph_oracle.hpp):
//   length(v) = sqrtf(((x*x + y*y) + z*z) + w*w), dot likewise;
//   fast_normalize(v) = v * (1 / sqrtf(dot(v, v)));
//   float4 / scalar is a true per-component division;
//   a double scalar times a float4 is rounded to float first (OpenCL converts
//   the scalar operand to the vector's element type);
//   unsuffixed floating literals are double (C++), as on an FP64 device.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>

typedef unsigned int uint;
typedef unsigned int cl_uint;
typedef unsigned char uchar;

#define __kernel
#define __global
#define __constant
#define __local
#define __private
#define __read_only
#define __write_only
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
typedef int sampler_t;
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_CLAMP_TO_EDGE 2
#define CLK_FILTER_NEAREST 0x10
#ifndef M_PI_F
#define M_PI_F 3.14159265358979323846f
#endif

struct float3 {
    float x, y, z;
};
struct int3 {
    int x, y, z;
};
// int2 with brace initialisation from any integer type (the kernels write
// `int2 p = {a_uint, b_uint}`).
struct int2 {
    int x, y;
    int2() {}
    template <class A, class B>
    int2(A a, B b) : x((int)a), y((int)b) {}
};
inline int2 make_int2(int a, int b) { return int2(a, b); }
inline int2 operator+(const int2& a, const int2& b) { return int2(a.x + b.x, a.y + b.y); }
inline int2 operator*(const int2& a, int s) { return int2(a.x * s, a.y * s); }
inline int2& operator+=(int2& a, const int2& b) {
    a.x += b.x;
    a.y += b.y;
    return a;
}

struct Swz3f {
    float v[3];
    operator float3() const { return float3{v[0], v[1], v[2]}; }
    Swz3f& operator=(const Swz3f& o) {
        v[0] = o.v[0]; v[1] = o.v[1]; v[2] = o.v[2];
        return *this;
    }
    Swz3f& operator=(const float3& o) {
        v[0] = o.x; v[1] = o.y; v[2] = o.z;
        return *this;
    }
    Swz3f& operator/=(float s) {
        v[0] = v[0] / s; v[1] = v[1] / s; v[2] = v[2] / s;
        return *this;
    }
    Swz3f& operator*=(float s) {
        v[0] = v[0] * s; v[1] = v[1] * s; v[2] = v[2] * s;
        return *this;
    }
};
struct Swz3i {
    int v[3];
    operator int3() const { return int3{v[0], v[1], v[2]}; }
    Swz3i& operator=(const Swz3i& o) {
        v[0] = o.v[0]; v[1] = o.v[1]; v[2] = o.v[2];
        return *this;
    }
    Swz3i& operator=(const int3& o) {
        v[0] = o.x; v[1] = o.y; v[2] = o.z;
        return *this;
    }
};

struct alignas(16) float4 {
    union {
        struct {
            float x, y, z, w;
        };
        Swz3f xyz;
    };
    float4() {}
    template <class A, class B, class C, class D>
    float4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
    float4(const float4& o) { std::memcpy(this, &o, 16); }
    float4& operator=(const float4& o) {
        std::memcpy(this, &o, 16);
        return *this;
    }
    float4& operator=(float s) {  // scalar assignment splats
        x = y = z = w = s;
        return *this;
    }
    float4& operator+=(const float4& o) {
        x = x + o.x; y = y + o.y; z = z + o.z; w = w + o.w;
        return *this;
    }
    float4& operator-=(const float4& o) {
        x = x - o.x; y = y - o.y; z = z - o.z; w = w - o.w;
        return *this;
    }
    float4& operator*=(float s) {
        x = x * s; y = y * s; z = z * s; w = w * s;
        return *this;
    }
    float4& operator/=(float s) {
        x = x / s; y = y / s; z = z / s; w = w / s;
        return *this;
    }
};
static_assert(sizeof(float4) == 16, "float4 size");

struct alignas(16) int4 {
    union {
        struct {
            int x, y, z, w;
        };
        Swz3i xyz;
        int2 xy;
        struct {
            int s0_, s1_, s2_, s3;
        };
    };
    int4() {}
    template <class A, class B, class C, class D>
    int4(A a, B b, C c, D d) : x((int)a), y((int)b), z((int)c), w((int)d) {}
    int4(const int4& o) { std::memcpy(this, &o, 16); }
    int4& operator=(const int4& o) {
        std::memcpy(this, &o, 16);
        return *this;
    }
};
static_assert(sizeof(int4) == 16, "int4 size");

inline float4 make_float4(float a, float b, float c, float d) {
    float4 r;
    r.x = a; r.y = b; r.z = c; r.w = d;
    return r;
}
inline float4 make_float4(const float3& v, float d) { return make_float4(v.x, v.y, v.z, d); }
inline int4 make_int4(int a, int b, int c, int d) {
    int4 r;
    r.x = a; r.y = b; r.z = c; r.w = d;
    return r;
}

inline float4 operator+(const float4& a, const float4& b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(const float4& a, const float4& b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator-(const float4& a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
inline float4 operator*(const float4& a, const float4& b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline float4 operator*(const float4& a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator*(float s, const float4& a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator*(const float4& a, double s) { return a * (float)s; }
inline float4 operator*(double s, const float4& a) { return (float)s * a; }
inline float4 operator*(const float4& a, int s) { return a * (float)s; }
inline float4 operator*(int s, const float4& a) { return (float)s * a; }
inline float4 operator/(const float4& a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4 operator/(const float4& a, double s) { return a / (float)s; }

inline int4 operator+(const int4& a, const int4& b) { return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
// convert_int4: the default conversion rounds toward zero.
inline int4 convert_int4(const float4& v) { return make_int4((int)v.x, (int)v.y, (int)v.z, (int)v.w); }

inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }
inline float3 operator+(const float3& a, const float3& b) { return float3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(const float3& a, const float3& b) { return float3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(const float3& a, float s) { return float3{a.x * s, a.y * s, a.z * s}; }
inline float3 operator*(const float3& a, double s) { return a * (float)s; }
inline float3 operator/(const float3& a, float s) { return float3{a.x / s, a.y / s, a.z / s}; }
inline float3 operator/(const float3& a, unsigned s) { return a / (float)s; }
// mix(x, y, a) = x + (y - x) * a (the OpenCL definition).
inline float3 mix(const float3& x, const float3& y, float a) { return x + (y - x) * a; }
inline float3 fast_normalize(const float3& v) { return v * (1.0f / std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z)); }
// native_divide: precision left to the implementation; here the correctly
// rounded quotient.
inline float native_divide(float a, float b) { return a / b; }
inline void vstore3(const float3& v, size_t i, float* p) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// image2d_t of float texels with CLK_ADDRESS_CLAMP_TO_EDGE reads.  A
// one-channel image (CL_R) stores .x and reads back (x, 0, 0, 1).
struct image2d_t {
    float4* data;
    int w, h, channels;
};
inline float4 read_imagef(const image2d_t& img, sampler_t, int2 p) {
    const int x = p.x < 0 ? 0 : (p.x >= img.w ? img.w - 1 : p.x);
    const int y = p.y < 0 ? 0 : (p.y >= img.h ? img.h - 1 : p.y);
    return img.data[(size_t)y * img.w + x];
}
inline void write_imagef(image2d_t& img, int2 p, const float4& v) {
    if (p.x < 0 || p.y < 0 || p.x >= img.w || p.y >= img.h) return;
    float4& t = img.data[(size_t)p.y * img.w + p.x];
    t = v;
    if (img.channels == 1) {
        t.y = 0.f;
        t.z = 0.f;
        t.w = 1.f;
    }
}
inline void write_imagef(image2d_t& img, int2 p, float v) { write_imagef(img, p, make_float4(v, v, v, v)); }

inline float dot(const float4& a, const float4& b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline float length(const float4& a) { return std::sqrt(dot(a, a)); }
// fast_normalize: OpenCL leaves its precision to the implementation; here
// v * (1 / sqrt(dot(v, v))), each operation correctly rounded.
inline float4 fast_normalize(const float4& v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }

namespace clshim {
struct WorkItem {
    size_t global_id, local_id, group_id, local_size, global_size;
    size_t global_id1, global_id2;  // dimensions 1 and 2 of a 3-D range
};
extern thread_local WorkItem g_item;
// Run f once per work-item of an NDRange of `global` items in groups of
// `local`, in group order; items of a group run as fibers so that barrier()
// works.  Items without barriers may use launch_flat (OpenMP over items).
void launch_groups(size_t global, size_t local, const std::function<void()>& f);
void barrier_impl();

template <class F>
inline void launch_flat(size_t global, size_t local, F&& f) {
#pragma omp parallel for schedule(static)
    for (long g = 0; g < (long)global; ++g) {
        g_item = WorkItem{(size_t)g, (size_t)g % local, (size_t)g / local, local, global};
        f();
    }
}
// A 3-D range of gx x gy x gz items without barriers (OpenMP over items).
template <class F>
inline void launch_flat3(size_t gx, size_t gy, size_t gz, F&& f) {
    const long total = (long)(gx * gy * gz);
#pragma omp parallel for schedule(static)
    for (long g = 0; g < total; ++g) {
        const size_t x = (size_t)g % gx, y = ((size_t)g / gx) % gy, z = (size_t)g / (gx * gy);
        g_item = WorkItem{x, 0, 0, 1, gx, y, z};
        f();
    }
}
}  // namespace clshim

inline size_t get_global_id(int d) {
    return d == 0 ? clshim::g_item.global_id : (d == 1 ? clshim::g_item.global_id1 : clshim::g_item.global_id2);
}
inline size_t get_local_id(int) { return clshim::g_item.local_id; }
inline size_t get_group_id(int) { return clshim::g_item.group_id; }
inline size_t get_local_size(int) { return clshim::g_item.local_size; }
inline size_t get_global_size(int) { return clshim::g_item.global_size; }
inline void barrier(int) { clshim::barrier_impl(); }

// Kernel::execute rounds the global size up to a multiple of the local size
// (rtpslib/opencl/Kernel.cpp:100-141).
inline size_t round_up(size_t n, size_t m) { return (n + m - 1) / m * m; }
