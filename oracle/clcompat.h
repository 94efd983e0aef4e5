// OpenCL C vocabulary in C++, so that Lensed's own device sources
// (objects/*.cl, kernel/*.cl and the program text generated by its
// src/kernel.c) compile on the host as the reference-built checker.
// TEST INFRASTRUCTURE ONLY (see oracle/build_ref.py).
//
// Work-items run one at a time with a local size of 1; ids come from
// thread-local state set by the harness, so barriers are no-ops.
// Elementary functions: REF_CR=1 evaluates them in double and rounds once
// to float (the strict FP32 semantics of the oracle); REF_CR=0 uses the C
// library's float functions.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstdint>

#ifndef REF_CR
#define REF_CR 1
#endif

typedef unsigned int uint;
typedef unsigned long ulong;

struct alignas(8) float2 {  // OpenCL alignment of float2
    union {
        struct {
            float x, y;
        };
        struct {
            float s0, s1;
        };
    };
    float2() = default;
    float2(int v) { x = y = (float)v; }
    float2(float v) { x = y = v; }
    float2(double v) { x = y = (float)v; }
    template <class A, class B>
    float2(A a, B b)
    {
        x = (float)a;
        y = (float)b;
    }
};

struct alignas(16) float4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float s0, s1, s2, s3;
        };
    };
    // halves, read-only (the generated text's .lo/.hi/.xy/.zw become calls)
    float2 lo() const { return float2(x, y); }
    float2 hi() const { return float2(z, w); }
    float2 xy() const { return float2(x, y); }
    float2 zw() const { return float2(z, w); }
    float4() = default;
    template <class A, class B, class C, class D>
    float4(A a, B b, C c, D d)
    {
        x = (float)a;
        y = (float)b;
        z = (float)c;
        w = (float)d;
    }
};

inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator-(float2 a) { return float2(-a.x, -a.y); }
inline float2 operator*(float2 a, float2 b) { return float2(a.x * b.x, a.y * b.y); }
inline float2 operator*(float s, float2 a) { return float2(s * a.x, s * a.y); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator/(float2 a, float s) { return float2(a.x / s, a.y / s); }
inline float2& operator+=(float2& a, float2 b) { return a = a + b; }
inline float2& operator-=(float2& a, float2 b) { return a = a - b; }
inline float2& operator*=(float2& a, float s) { return a = a * s; }
inline float4 operator*(float s, float4 a) { return float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator/(float4 a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float length(float2 a) { return std::sqrt(dot(a, a)); }
inline float2 normalize(float2 a)
{
    if (a.x == 0 && a.y == 0) return a;
    float l = length(a);
    return float2(a.x / l, a.y / l);
}

#if REF_CR
#define REF_F1(name) \
    inline float name(float x) { return (float)std::name((double)x); }
inline float pow_f(float x, float y) { return (float)std::pow((double)x, (double)y); }
inline float atan2_f(float y, float x) { return (float)std::atan2((double)y, (double)x); }
#else
#define REF_F1(name) \
    inline float name(float x) { return std::name(x); }
inline float pow_f(float x, float y) { return std::pow(x, y); }
inline float atan2_f(float y, float x) { return std::atan2(y, x); }
#endif
namespace refmath {
REF_F1(exp)
REF_F1(log)
REF_F1(sin)
REF_F1(cos)
REF_F1(atan)
REF_F1(atanh)
REF_F1(tgamma)
}  // namespace refmath
using refmath::atan;
using refmath::atanh;
using refmath::cos;
using refmath::exp;
using refmath::log;
using refmath::sin;
using refmath::tgamma;
inline float sqrt(float x) { return std::sqrt(x); }
inline float powr(float x, float y) { return pow_f(x, y); }
inline float pow(float x, float y) { return pow_f(x, y); }
inline float atan2(float y, float x) { return atan2_f(y, x); }
inline float sincos(float x, float* c)
{
    *c = cos(x);
    return sin(x);
}

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int mad24(int a, int b, int c) { return a * b + c; }

// a pointer that converts to any object pointer: stands in for the
// generated code's (local void*)(data + offset) arguments
struct lg_anyptr {
    void* p;
    template <class T>
    lg_anyptr(T* q) : p((void*)q)
    {
    }
    template <class T>
    operator T*() const
    {
        return (T*)p;
    }
};

// work-item state, set by the harness before each call
extern thread_local size_t ref_gid[2], ref_grp[2];
inline size_t get_global_id(int d) { return ref_gid[d]; }
inline size_t get_group_id(int d) { return ref_grp[d]; }
inline size_t get_local_id(int) { return 0; }
inline size_t get_local_size(int) { return 1; }
#define CLK_LOCAL_MEM_FENCE 0
inline void barrier(int) {}

// address-space qualifiers and the kernel keyword
#define kernel
#define global
#define local
#define constant const
#define this self_
