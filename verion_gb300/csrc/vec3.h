// Three-component float vector with the component-wise semantics of Slang's float3.
// Every operation is a plain IEEE single-precision operation in a fixed order, so host and device
// builds without FMA contraction agree bit for bit. Vector / scalar divides each component
// (it does not multiply by a reciprocal).
#pragma once
#include "vg_math.h"

struct V3 {
    float x, y, z;
};

VG_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
VG_HD V3 v3(float s) { return V3{s, s, s}; }
VG_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
VG_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
VG_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
VG_HD V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
VG_HD V3 operator+(V3 a, float s) { return V3{a.x + s, a.y + s, a.z + s}; }
VG_HD V3 operator+(float s, V3 a) { return V3{s + a.x, s + a.y, s + a.z}; }
VG_HD V3 operator-(float s, V3 a) { return V3{s - a.x, s - a.y, s - a.z}; }
VG_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
VG_HD V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
VG_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
VG_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
VG_HD V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
VG_HD V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
VG_HD V3& operator*=(V3& a, float s) { a = a * s; return a; }
VG_HD V3& operator/=(V3& a, float s) { a = a / s; return a; }
VG_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VG_HD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
VG_HD float length(V3 a) { return sqrtf(dot(a, a)); }
VG_HD V3 normalize(V3 a)
{
    float inv = 1.0f / sqrtf(dot(a, a));
    return a * inv;
}
VG_HD float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
VG_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
VG_HD float saturatef(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
VG_HD float lerpf(float a, float b, float t) { return a + t * (b - a); }
VG_HD V3 lerp3(V3 a, V3 b, float t) { return a + t * (b - a); }
VG_HD bool bad3(V3 a)
{
    return isnan(a.x) || isnan(a.y) || isnan(a.z) || isinf(a.x) || isinf(a.y) || isinf(a.z);
}
