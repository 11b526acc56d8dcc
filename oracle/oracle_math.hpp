// TEST INFRASTRUCTURE — the parity oracle, not the product. Only tests/, the smoke check and the
// benchmark's CPU-baseline leg load it.
//
// f32 vector arithmetic in the operation order of glam 0.33 (the reference's math crate, via
// bevy_math 0.20; Cargo.lock:3006) as its call sites use it, the bake's RNG and its
// transcendental policy. Every formula is written so that, compiled with -ffp-contract=off and
// without -ffast-math, it rounds exactly like the reference's Rust (which never contracts a*b+c).
//
// glam is not vendored under the reference, so its operation orders are restated from its
// published behaviour and pinned only by the reference's tolerance tests (parity at this
// boundary is unpinned): dot = (x*x' + y*y') + z*z'; cross(a, b).x = a.y*b.z - b.y*a.z;
// normalize(v) = v * (1 / sqrt(dot(v, v))); any_orthonormal_pair is Duff et al. 2017
// ("Building an Orthonormal Basis, Revisited").
//
// Transcendentals (sin, cos, tan, exp of f32 arguments) are evaluated in binary64 and rounded
// once to binary32: Cody–Waite reduction by pi/2 (Cody & Waite 1980) and the Taylor series of
// sin/cos, so both this oracle and the CUDA kernels produce the correctly rounded f32 in all but
// ~1e-8 of arguments and agree with each other bit for bit. The reference calls the platform
// libm (src/bake/mesh_texels.rs:121, random.rs:26, sun.rs:41, light_shape.rs:55,
// bounce_map.rs:146), whose f32 results are within one ulp. Its one arccosine, the angle of
// glam's slerp (src/bake/bounce.rs:270), is glam's own binary32 polynomial, restated exactly
// (acos_approx, oracle_bounce.hpp).
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle {

struct V2 {
    float x, y;
};
struct V3 {
    float x, y, z;
};

inline V2 v2(float x, float y) { return V2{x, y}; }
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline bool operator==(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool is_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator*(V2 a, float s) { return {a.x * s, a.y * s}; }

inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline float length_squared(V3 a) { return dot(a, a); }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline float length_recip(V3 a) { return 1.0f / length(a); }
inline V3 normalize(V3 a) { return a * length_recip(a); }
inline bool finite_positive(float r) { return std::isfinite(r) && r > 0.0f; }
inline V3 normalize_or(V3 a, V3 fallback) {
    float r = length_recip(a);
    return finite_positive(r) ? a * r : fallback;
}
inline V3 normalize_or_zero(V3 a) { return normalize_or(a, V3{0, 0, 0}); }
// try_normalize(): nullopt as `ok == false`.
inline V3 try_normalize(V3 a, bool &ok) {
    float r = length_recip(a);
    ok = finite_positive(r);
    return ok ? a * r : V3{0, 0, 0};
}
inline float distance_squared(V3 a, V3 b) { return length_squared(a - b); }
// Rust f32::min / f32::max: the non-NaN operand when one is NaN.
inline float fmin_r(float a, float b) { return std::fmin(a, b); }
inline float fmax_r(float a, float b) { return std::fmax(a, b); }
inline V3 vmin(V3 a, V3 b) { return {fmin_r(a.x, b.x), fmin_r(a.y, b.y), fmin_r(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {fmax_r(a.x, b.x), fmax_r(a.y, b.y), fmax_r(a.z, b.z)}; }
inline V2 vmin2(V2 a, V2 b) { return {fmin_r(a.x, b.x), fmin_r(a.y, b.y)}; }
inline V2 vmax2(V2 a, V2 b) { return {fmax_r(a.x, b.x), fmax_r(a.y, b.y)}; }
inline float max_element(V3 a) { return fmax_r(fmax_r(a.x, a.y), a.z); }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
// geometry.rs:138-140
inline bool approx_eq(V3 a, V3 b, float eps) { return max_element(vabs(a - b)) < eps; }
inline bool v3_finite(V3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

// Rust `f as u32`: saturating, NaN to 0.
inline uint32_t f2u_sat(float f) {
    if (!(f > 0.0f)) return 0u;  // NaN, negative, zero
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
// Rust `f as u8` / `as i8`: saturating.
inline uint8_t f2u8_sat(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 255.0f) return 255;
    return (uint8_t)f;
}
inline int8_t f2i8_sat(float f) {
    if (std::isnan(f)) return 0;
    if (f <= -128.0f) return -128;
    if (f >= 127.0f) return 127;
    return (int8_t)f;
}
// f32::clamp (NaN stays NaN)
inline float clampf(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}

// Duff, Burgess, Christensen, Hery, Kensler, Liani, Villemin: "Building an Orthonormal Basis,
// Revisited" (JCGT 2017), as glam's Vec3::any_orthonormal_pair applies it.
inline void any_orthonormal_pair(V3 n, V3 &a_out, V3 &b_out) {
    float sign = std::signbit(n.z) ? -1.0f : 1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    a_out = V3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    b_out = V3{b, sign + n.y * n.y * a, -n.y};
}

// Quat * Vec3 as glam evaluates it: v(w² − |b|²) + b(2 v·b) + (b × v)(2w).
inline V3 quat_rotate(const float q[4], V3 v) {
    V3 b{q[0], q[1], q[2]};
    float w = q[3];
    float b2 = dot(b, b);
    return (v * (w * w - b2) + b * (dot(v, b) * 2.0f)) + cross(b, v) * (w * 2.0f);
}

// ---- transcendentals: binary64 evaluation, one rounding -------------------------------------
// pi/2 = PIO2_HI + PIO2_LO, PIO2_HI holding the leading 33 bits (so k * PIO2_HI is exact).
constexpr double PIO2_HI = 1.5707963267341256;       // 0x1.921fb54400000p+0
constexpr double PIO2_LO = 6.077100506506192e-11;    // 0x1.0b4611a626331p-34
constexpr double TWO_OVER_PI = 0.6366197723675814;
constexpr double PI_D = 3.141592653589793;

// sin and cos of r, |r| <= pi/4, by their Taylor series (coefficients (-1)^n/(2n+1)!, (-1)^n/(2n)!).
inline void sincos_kernel(double r, double &s, double &c) {
    double r2 = r * r;
    double ps = -3.868170170630684e-23;
    ps = ps * r2 + 1.9572941063391263e-20;
    ps = ps * r2 + -8.22063524662433e-18;
    ps = ps * r2 + 2.8114572543455206e-15;
    ps = ps * r2 + -7.647163731819816e-13;
    ps = ps * r2 + 1.6059043836821613e-10;
    ps = ps * r2 + -2.505210838544172e-08;
    ps = ps * r2 + 2.7557319223985893e-06;
    ps = ps * r2 + -0.0001984126984126984;
    ps = ps * r2 + 0.008333333333333333;
    ps = ps * r2 + -0.16666666666666666;
    s = r + r * (r2 * ps);
    double pc = -8.896791392450574e-22;
    pc = pc * r2 + 4.110317623312165e-19;
    pc = pc * r2 + -1.5619206968586225e-16;
    pc = pc * r2 + 4.779477332387385e-14;
    pc = pc * r2 + -1.1470745597729725e-11;
    pc = pc * r2 + 2.08767569878681e-09;
    pc = pc * r2 + -2.755731922398589e-07;
    pc = pc * r2 + 2.48015873015873e-05;
    pc = pc * r2 + -0.001388888888888889;
    pc = pc * r2 + 0.041666666666666664;
    pc = pc * r2 + -0.5;
    c = 1.0 + r2 * pc;
}

// sin and cos of a binary64 argument of modest size (|x| < 2^20).
inline void sincos_d(double x, double &s, double &c) {
    double k = std::nearbyint(x * TWO_OVER_PI);
    double r = (x - k * PIO2_HI) - k * PIO2_LO;
    double sr, cr;
    sincos_kernel(r, sr, cr);
    long q = (long)k & 3;
    switch (q) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

inline void sincos_f(float x, float &s, float &c) {
    if (!std::isfinite(x)) {
        s = c = NAN;
        return;
    }
    double sd, cd;
    sincos_d((double)x, sd, cd);
    s = (float)sd;
    c = (float)cd;
}
inline float sin_f(float x) { float s, c; sincos_f(x, s, c); return s; }
inline float cos_f(float x) { float s, c; sincos_f(x, s, c); return c; }
inline float tan_f(float x) {
    if (!std::isfinite(x)) return NAN;
    double s, c;
    sincos_d((double)x, s, c);
    return (float)(s / c);
}

inline float exp_f(float x) { return (float)std::exp((double)x); }

constexpr float TAU_F = 6.28318530717958647692f;    // f32 TAU
constexpr float PI_F = 3.14159265358979323846f;     // f32 PI
constexpr float FRAC_PI_4_F = 0.78539816339744830962f;

// ---- RNG: SplitMix64 (src/effects/rng.rs:10-15), PCG32 XSH-RR (rng.rs:35-71),
// keyed streams (src/bake/random.rs:9-19). ----------------------------------------------------
inline uint64_t splitmix64(uint64_t v) {
    v += 0x9e3779b97f4a7c15ull;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}
inline uint64_t key_seed(const uint64_t *parts, int n) {
    uint64_t acc = 0x0b4ce5eed0000000ull;
    for (int i = 0; i < n; ++i) acc = splitmix64(acc ^ splitmix64(parts[i]));
    return acc;
}
struct Rng {
    uint64_t state, increment;
    uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + increment;
        uint32_t xorshifted = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
    }
    float next_f32() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
};
inline Rng rng_new(uint64_t seed, uint64_t stream) {
    Rng r{0, (stream << 1) | 1};
    r.next_u32();
    r.state += seed;
    r.next_u32();
    return r;
}
inline Rng stream(const uint64_t *parts, int n) {
    uint64_t s = key_seed(parts, n);
    return rng_new(s, (s << 17) | (s >> 47));
}
// random.rs:22-27
inline V3 on_unit_sphere(Rng &rng) {
    float z = rng.next_f32() * 2.0f - 1.0f;
    float angle = rng.next_f32() * TAU_F;
    float r = std::sqrt(fmax_r(1.0f - z * z, 0.0f));
    float s, c;
    sincos_f(angle, s, c);
    return V3{r * c, r * s, z};
}

// ---- precision modes ------------------------------------------------------------------------
// F32 restates the reference's binary32 arithmetic. REFINED restates the GPU library's refined
// form: binary32, except that ray/triangle tests landing within eps of a boundary are re-run
// in binary64 and soft-visibility weights and bounce gathers use Kahan sums. F64 is the FP64
// oracle: every ray/triangle test, the soft-visibility and bounce sums and the fractions they
// give in binary64, over the same binary32 samples (origins, directions, weights, integrands),
// so it measures the predicates and the accumulation, not the sampling. REFINED_BOUNCE restates
// the library's bounce-refined form: F32 everywhere but in the bounce stages (photon cubes and
// gathers), which run as REFINED.
enum Precision : uint32_t { PREC_F32 = 0, PREC_REFINED = 1, PREC_F64 = 2, PREC_REFINED_BOUNCE = 3 };
struct PrecisionMode {
    Precision mode = PREC_F32;    // outside the bounce stages
    Precision bounce = PREC_F32;  // inside them
    float eps = 1.0e-5f, eps2 = 1.0e-10f;
};
inline PrecisionMode &precision() {
    static PrecisionMode p;
    return p;
}
// Whether this thread is inside a bounce stage (BounceScope), and the mode in force there.
inline bool &in_bounce_stage() {
    static thread_local bool on = false;
    return on;
}
inline Precision active_mode() { return in_bounce_stage() ? precision().bounce : precision().mode; }
struct BounceScope {
    bool was;
    BounceScope() : was(in_bounce_stage()) { in_bounce_stage() = true; }
    ~BounceScope() { in_bounce_stage() = was; }
};

struct D3 {
    double x, y, z;
};
inline D3 widen(V3 a) { return D3{(double)a.x, (double)a.y, (double)a.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }

// A running sum of binary32 terms in the active mode: plain binary32, Kahan (REFINED) or
// binary64 (F64).
struct Acc {
    float s = 0.0f, c = 0.0f;
    double d = 0.0;
    void add(float x) {
        switch (active_mode()) {
        case PREC_F64: d += (double)x; break;
        case PREC_REFINED: {
            float y = x - c;
            float t = s + y;
            c = (t - s) - y;
            s = t;
            break;
        }
        default: s = s + x;
        }
    }
    double value() const { return active_mode() == PREC_F64 ? d : (double)s; }
};
struct Acc3 {
    Acc x, y, z;
    void add(V3 v) {
        x.add(v.x);
        y.add(v.y);
        z.add(v.z);
    }
    // sum * scale / n: binary32 in F32/REFINED (the reference's `sum * intensity / samples`),
    // binary64 rounded once in F64
    V3 mean(float scale, uint32_t n) const {
        if (active_mode() == PREC_F64)
            return V3{(float)(x.d * scale / n), (float)(y.d * scale / n), (float)(z.d * scale / n)};
        return V3{x.s, y.s, z.s} * scale / (float)n;
    }
};

}  // namespace oracle
