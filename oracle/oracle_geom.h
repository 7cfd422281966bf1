// oracle_geom.h — float32 vector helpers for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY. The oracle is the checker for the CUDA engine:
// nothing in the product links or calls it.
//
// Every operation is spelled out in a fixed left-to-right order and the
// oracle is compiled with -ffp-contract=off, so a multiply followed by an
// add is never fused. The CUDA kernels compile the same expressions with
// --fmad=false; together this makes float32 results comparable bit for bit.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

static inline f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
// dot(a, b) = (a.x b.x + a.y b.y) + a.z b.z
static inline float dot(f3 a, f3 b) {
  float r = a.x * b.x;
  r = r + a.y * b.y;
  r = r + a.z * b.z;
  return r;
}
static inline f3 cross(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline f3 xyz(f4 p) { return mk3(p.x, p.y, p.z); }
static inline float vmin(float a, float b) { return b < a ? b : a; }
static inline float vmax(float a, float b) { return b > a ? b : a; }
static inline f3 vmin3(f3 a, f3 b) { return mk3(vmin(a.x, b.x), vmin(a.y, b.y), vmin(a.z, b.z)); }
static inline f3 vmax3(f3 a, f3 b) { return mk3(vmax(a.x, b.x), vmax(a.y, b.y), vmax(a.z, b.z)); }
static inline float comp(f3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

}  // namespace orc
