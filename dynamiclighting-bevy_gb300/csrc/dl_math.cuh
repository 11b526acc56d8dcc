// f32 arithmetic of the bake in the reference's operation order, for host and device.
//
// The library is compiled with --fmad=false (device) and -ffp-contract=off (host), so every
// a*b+c below rounds twice exactly like the reference's Rust (src/bake/*.rs), which never
// contracts. Vector conventions follow glam 0.33 as the reference uses it:
//   dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a, b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
// Transcendentals of f32 arguments: the binary64 evaluation (Cody–Waite reduction by pi/2 and
// Taylor series, rounded once) is the definition host and device share. On the device, sin/cos
// first run in double-float binary32 arithmetic (error-free sums and products, Dekker 1971) to
// about 2^-40 and keep that result only when Ziv's rounding test shows it rounds to the same
// binary32 as the exact value; otherwise the binary64 path decides, so both give one answer.
// acos is glam's acos_approx, a binary32 polynomial (below), as the reference's slerp takes it.
#pragma once

#include <cstdint>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define DL_HD __host__ __device__ __forceinline__
#define DL_HD_OUTLINE static __host__ __device__ __noinline__  // one shared copy per unit
#else
#define DL_HD inline
#define DL_HD_OUTLINE inline
#endif

namespace dl {

struct f2 {
    float x, y;
};
struct f3 {
    float x, y, z;
};

DL_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
DL_HD f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
DL_HD f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
DL_HD f3 neg(f3 a) { return f3{-a.x, -a.y, -a.z}; }
DL_HD f3 scale(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
DL_HD f3 divs(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
DL_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DL_HD f3 cross(f3 a, f3 b) { return f3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
DL_HD bool is_zero(f3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
DL_HD float length_sq(f3 a) { return dot(a, a); }
DL_HD float length(f3 a) { return sqrtf(dot(a, a)); }
DL_HD bool finite_pos(float r) { return isfinite(r) && r > 0.0f; }
DL_HD f3 normalize(f3 a) { return scale(a, 1.0f / length(a)); }
DL_HD f3 normalize_or(f3 a, f3 fb) {
    float r = 1.0f / length(a);
    return finite_pos(r) ? scale(a, r) : fb;
}
DL_HD f3 normalize_or_zero(f3 a) { return normalize_or(a, f3{0.0f, 0.0f, 0.0f}); }
DL_HD f3 try_normalize(f3 a, bool &ok) {
    float r = 1.0f / length(a);
    ok = finite_pos(r);
    return ok ? scale(a, r) : f3{0.0f, 0.0f, 0.0f};
}
// binary64 vectors for the refined form's ray/triangle re-test (same operation order as f3)
struct d3 {
    double x, y, z;
};
DL_HD d3 widen(f3 a) { return d3{(double)a.x, (double)a.y, (double)a.z}; }
DL_HD d3 sub(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
DL_HD double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DL_HD d3 cross(d3 a, d3 b) { return d3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }

// A binary32 running sum; KAHAN selects compensated summation (Kahan 1965), which the refined
// form uses for soft-visibility weights and bounce gathers.
template <bool KAHAN>
struct FSum {
    float s = 0.0f, c = 0.0f;
    DL_HD void add(float x) {
        if (KAHAN) {
            float y = x - c;
            float t = s + y;
            c = (t - s) - y;
            s = t;
        } else {
            s = s + x;
        }
    }
};
template <bool KAHAN>
struct FSum3 {
    FSum<KAHAN> x, y, z;
    DL_HD void add(f3 v) {
        x.add(v.x);
        y.add(v.y);
        z.add(v.z);
    }
    DL_HD f3 value() const { return f3{x.s, y.s, z.s}; }
};

// binary32 -> binary16 bits, round to nearest even (IEEE 754; the distance cubes' f16 packing,
// src/bake/distance_cubes.rs:23-26)
DL_HD uint32_t f16_bits(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, a = x & 0x7FFFFFFFu;
    if (a > 0x7F800000u) return sign | 0x7E00u | ((a >> 13) & 0x3FFu);  // NaN
    if (a >= 0x477FF000u) return sign | 0x7C00u;                      // 65520 and up: infinity
    int e = (int)(a >> 23) - 127;
    if (e >= -14) {
        uint32_t h = ((uint32_t)(e + 15) << 10) | ((a >> 13) & 0x3FFu), rest = a & 0x1FFFu;
        if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) ++h;
        return sign | h;
    }
    if (a == 0) return sign;
    int shift = -e - 1;  // half subnormals: value / 2^-24 = mantissa * 2^(e + 1)
    if (shift > 24) return sign;
    uint32_t mant = (a & 0x7FFFFFu) | 0x800000u;
    uint32_t q = mant >> shift, rest = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if (rest > half || (rest == half && (q & 1u))) ++q;
    return sign | q;
}

DL_HD float fminr(float a, float b) { return fminf(a, b); }
DL_HD float fmaxr(float a, float b) { return fmaxf(a, b); }
DL_HD f3 vmin(f3 a, f3 b) { return f3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
DL_HD f3 vmax(f3 a, f3 b) { return f3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
DL_HD float max_elem(f3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
DL_HD bool approx_eq(f3 a, f3 b, float eps) {
    f3 d = sub(a, b);
    return fmaxf(fmaxf(fabsf(d.x), fabsf(d.y)), fabsf(d.z)) < eps;
}
DL_HD float clampf(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}
// Rust `as u32` / `as u8` / `as i8`: saturating, NaN to 0.
DL_HD uint32_t f2u(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
DL_HD uint32_t f2u8(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 255.0f) return 255u;
    return (uint32_t)f;
}
DL_HD int f2i8(float f) {
    if (isnan(f)) return 0;
    if (f <= -128.0f) return -128;
    if (f >= 127.0f) return 127;
    return (int)f;
}

// Orthonormal basis around a unit vector (Duff et al., JCGT 2017), as glam's
// Vec3::any_orthonormal_pair evaluates it.
DL_HD void ortho_pair(f3 n, f3 &a, f3 &b) {
    float sign = signbit(n.z) ? -1.0f : 1.0f;
    float k = -1.0f / (sign + n.z);
    float m = n.x * n.y * k;
    a = f3{1.0f + sign * n.x * n.x * k, sign * m, -sign * n.x};
    b = f3{m, sign + n.y * n.y * k, -n.y};
}

// Quaternion (x, y, z, w) times vector: v(w^2 - |q|^2) + q(2 v.q) + (q x v)(2w).
DL_HD f3 quat_rotate(const float q[4], f3 v) {
    f3 b{q[0], q[1], q[2]};
    float w = q[3];
    float b2 = dot(b, b);
    return add(add(scale(v, w * w - b2), scale(b, dot(v, b) * 2.0f)), scale(cross(b, v), w * 2.0f));
}

// ---- transcendentals ---------------------------------------------------------------------------
// pi/2 split for Cody–Waite reduction: the high part holds 33 significant bits.
constexpr double kPio2Hi = 1.5707963267341256;     // 0x1.921fb54400000p+0
constexpr double kPio2Lo = 6.077100506506192e-11;  // 0x1.0b4611a626331p-34
constexpr double kTwoOverPi = 0.6366197723675814;
constexpr double kPi = 3.141592653589793;

// Taylor series of sin and cos on |r| <= pi/4 (coefficients (-1)^n/(2n+1)! and (-1)^n/(2n)!).
DL_HD void sincos_poly(double r, double &s, double &c) {
    double r2 = r * r;
    double p = -3.868170170630684e-23;
    p = p * r2 + 1.9572941063391263e-20;
    p = p * r2 + -8.22063524662433e-18;
    p = p * r2 + 2.8114572543455206e-15;
    p = p * r2 + -7.647163731819816e-13;
    p = p * r2 + 1.6059043836821613e-10;
    p = p * r2 + -2.505210838544172e-08;
    p = p * r2 + 2.7557319223985893e-06;
    p = p * r2 + -0.0001984126984126984;
    p = p * r2 + 0.008333333333333333;
    p = p * r2 + -0.16666666666666666;
    s = r + r * (r2 * p);
    double q = -8.896791392450574e-22;
    q = q * r2 + 4.110317623312165e-19;
    q = q * r2 + -1.5619206968586225e-16;
    q = q * r2 + 4.779477332387385e-14;
    q = q * r2 + -1.1470745597729725e-11;
    q = q * r2 + 2.08767569878681e-09;
    q = q * r2 + -2.755731922398589e-07;
    q = q * r2 + 2.48015873015873e-05;
    q = q * r2 + -0.001388888888888889;
    q = q * r2 + 0.041666666666666664;
    q = q * r2 + -0.5;
    c = 1.0 + r2 * q;
}
DL_HD void sincos_d(double x, double &s, double &c) {
    double k = nearbyint(x * kTwoOverPi);
    double r = (x - k * kPio2Hi) - k * kPio2Lo;
    double sr, cr;
    sincos_poly(r, sr, cr);
    switch ((long long)k & 3) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}
// ---- binary32 double-float path with a rounding test ---------------------------------------
// GB300 runs binary64 at a small fraction of its binary32 rate, so sin/cos first run in
// double-float binary32 arithmetic (error-free sums and FMA products; Dekker 1971, Knuth TAOCP
// 4.2.2) to within 2^-40 of the true value, and the result is kept only when the rounding test
// of Ziv's strategy (Ziv 1991) proves it is the correctly rounded binary32 value; otherwise the
// binary64 path below decides. Either way the value equals what the binary64 path returns.
struct FF {
    float h, l;
};
DL_HD FF ff_two_sum(float a, float b) {
    float s = a + b;
    float bb = s - a;
    return FF{s, (a - (s - bb)) + (b - bb)};
}
DL_HD FF ff_fast_sum(float a, float b) {
    float s = a + b;
    return FF{s, b - (s - a)};
}
DL_HD FF ff_mul(FF a, FF b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = e + (a.h * b.l + a.l * b.h);
    return ff_fast_sum(p, e);
}
DL_HD FF ff_add(FF a, FF b) {
    FF s = ff_two_sum(a.h, b.h);
    return ff_fast_sum(s.h, s.l + (a.l + b.l));
}
DL_HD FF ff_add_f(FF a, float b) {
    FF s = ff_two_sum(a.h, b);
    return ff_fast_sum(s.h, s.l + a.l);
}
DL_HD FF ff_neg(FF a) { return FF{-a.h, -a.l}; }

// sin(r) and cos(r), |r| <= pi/4, r = rh + rl: Taylor coefficients as binary32 pairs (hi + lo =
// (-1)^n/(2n+1)! or (-1)^n/(2n)! to 48 bits) for the leading terms, single binary32 for the tail
// terms whose share of the result is below 2^-17.
DL_HD FF ff_sin_poly(FF r, FF r2) {
    float z = r2.h;
    float ts = 2.7557318844628753e-06f + z * (-2.5052107943679403e-08f + z * (1.6059044372074283e-10f +
                                                                            z * -7.647163609812713e-13f));
    FF p = ff_add_f(FF{-0.00019841270113829523f, 2.725596874933456e-12f}, z * ts);
    p = ff_add(FF{0.008333333767950535f, -4.34617203337595e-10f}, ff_mul(r2, p));
    p = ff_add(FF{-0.1666666716337204f, 4.967053879312289e-09f}, ff_mul(r2, p));
    return ff_add(r, ff_mul(ff_mul(r, r2), p));
}
DL_HD FF ff_cos_poly(FF r2) {
    float z = r2.h;
    float tc = 2.4801587642286904e-05f + z * (-2.755731998149713e-07f + z * (2.0876755879584152e-09f +
                                                                          z * -1.147074536050896e-11f));
    FF q = ff_add_f(FF{-0.0013888889225199819f, 3.3631094437103215e-11f}, z * tc);
    q = ff_add(FF{0.0416666679084301f, -1.2417634698280722e-09f}, ff_mul(r2, q));
    q = ff_add_f(ff_mul(r2, q), -0.5f);
    return ff_add_f(ff_mul(r2, q), 1.0f);
}
DL_HD void ff_sincos_poly(FF r, FF &s, FF &c) {
    FF r2 = ff_mul(r, r);
    s = ff_sin_poly(r, r2);
    c = ff_cos_poly(r2);
}
// Ziv's rounding test: true when every value within 2^-36 relative of h + l rounds to h. The
// gaps to the neighbouring binary32 values come from h's exponent bits: 2^(e-23) away from zero,
// and half that towards zero when h is a power of two (its binade's lower edge).
DL_HD bool ff_rounds_to(FF v, float &out) {
    float a = fabsf(v.h);
    if (!(a >= 1.0e-30f && a < 1.0e30f)) return false;
    uint32_t bits;
    memcpy(&bits, &a, 4);
    const uint32_t pow2 = bits & 0x7F800000u;
    float ulp;
    memcpy(&ulp, &pow2, 4);
    ulp = ulp * 1.1920928955078125e-07f;  // 2^-23: exact, the result stays normal for a >= 1e-30
    const float away = ulp, toward = (bits & 0x007FFFFFu) ? ulp : 0.5f * ulp;
    const float up = v.h > 0.0f ? away : toward, down = v.h > 0.0f ? toward : away;
    float err = a * 1.4551915228366852e-11f;  // 2^-36, far above the path's 2^-40 error bound
    if (v.l + err < 0.5f * up && v.l - err > -0.5f * down) {
        out = v.h;
        return true;
    }
    return false;
}

// pi/2 as C1 + C2 + C3 in binary32, C1 and C2 holding 21 significant bits so k * C1 and k * C2
// are exact for the small quadrant counts k of the bake's angles (|x| < 16).
constexpr float kPio2F1 = 1.570796012878418f;      // 0x1.921fb0p+0
constexpr float kPio2F2 = 3.139164164167596e-07f;  // 0x1.5110b0p-22
constexpr float kPio2F3 = 6.223371969669989e-14f;  // 0x1.184698p-44

// The binary64 path of sincos_f and sin_f, out of line: it runs for a small share of arguments,
// so one shared copy keeps the call sites' code (and the instruction cache they need) small.
DL_HD_OUTLINE void sincos_rounded_b64(float x, float &s, float &c) {
    double sd, cd;
    sincos_d((double)x, sd, cd);
    s = (float)sd;
    c = (float)cd;
}

DL_HD void sincos_f(float x, float &s, float &c) {
    if (!isfinite(x)) {
        s = c = NAN;
        return;
    }
    if (x != 0.0f && fabsf(x) < 16.0f) {
        // Cody–Waite reduction in binary32: x - k*C1 is exact (Sterbenz), the k*C2 term enters
        // through an error-free sum, k*C3 through the low word.
        float k = rintf(x * 0.6366197466850281f);
        FF r = ff_two_sum(x - k * kPio2F1, -(k * kPio2F2));
        r = ff_fast_sum(r.h, r.l - k * kPio2F3);
        // k = 0 needs no reduction; near-multiples of pi/2 (|r| <= 2^-16) go to binary64
        if (k == 0.0f || fabsf(r.h) > 1.52587890625e-05f) {
            FF sv, cv;
            ff_sincos_poly(r, sv, cv);
            FF so, co;
            switch ((int)k & 3) {
                case 0: so = sv; co = cv; break;
                case 1: so = cv; co = ff_neg(sv); break;
                case 2: so = ff_neg(sv); co = ff_neg(cv); break;
                default: so = ff_neg(cv); co = sv; break;
            }
            if (ff_rounds_to(so, s) && ff_rounds_to(co, c)) return;
        }
    }
    // binary64 path: Cody–Waite reduction and Taylor series in binary64, one rounding
    sincos_rounded_b64(x, s, c);
}
// sin alone: the reduction of sincos_f and only the polynomial the quadrant needs (sin of the
// reduced argument for even quadrants, cos for odd ones), its own rounding test, the same
// binary64 fallback.
DL_HD float sin_f(float x) {
    if (isfinite(x) && x != 0.0f && fabsf(x) < 16.0f) {
        float k = rintf(x * 0.6366197466850281f);
        FF r = ff_two_sum(x - k * kPio2F1, -(k * kPio2F2));
        r = ff_fast_sum(r.h, r.l - k * kPio2F3);
        if (k == 0.0f || fabsf(r.h) > 1.52587890625e-05f) {
            const int q = (int)k & 3;
            FF r2 = ff_mul(r, r);
            FF v = (q & 1) ? ff_cos_poly(r2) : ff_sin_poly(r, r2);
            if (q & 2) v = ff_neg(v);
            float s;
            if (ff_rounds_to(v, s)) return s;
        }
    }
    if (!isfinite(x)) return NAN;
    float s, c;
    sincos_rounded_b64(x, s, c);
    return s;
}
// sin_f as one shared out-of-line copy, for call sites that take several sines in a row (the
// bounce slerp's three).
DL_HD_OUTLINE float sin_f_outline(float x) { return sin_f(x); }
DL_HD float tan_f(float x) {
    if (!isfinite(x)) return NAN;
    double s, c;
    sincos_d((double)x, s, c);
    return (float)(s / c);
}
// glam's acos_approx (the angle of Vec3::slerp): Abramowitz & Stegun 4.4.46 (Hastings'
// 7-degree polynomial; DirectXMath's XMScalarACos has the same coefficients), in binary32 with
// no fused operations: sqrt(1 - |x|) * p(|x|) by Horner's rule, and pi minus it for x < 0.
DL_HD float acos_approx(float v) {
    const bool nonnegative = v >= 0.0f;
    const float x = fabsf(v);
    float omx = 1.0f - x;
    if (omx < 0.0f) omx = 0.0f;
    const float root = sqrtf(omx);
    float r = -0.0012624911f;  // (the library is compiled with --fmad=false: no contraction)
    r = r * x + 0.0066700901f;
    r = r * x - 0.0170881256f;
    r = r * x + 0.0308918810f;
    r = r * x - 0.0501743046f;
    r = r * x + 0.0889789874f;
    r = r * x - 0.2145988016f;
    r = r * x + 1.5707963050f;
    r = r * root;
    return nonnegative ? r : 3.14159265358979323846f - r;
}
constexpr float kTau = 6.28318530717958647692f;
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kFracPi4 = 0.78539816339744830962f;
constexpr float kNdotlTolerance = -0.1f;  // mesh_bake.rs:25
constexpr float kRayOffset = 0.001f;      // mesh_bake.rs:27
constexpr float kEndGap = 1.0e-3f;        // area.rs:33

// ---- RNG: SplitMix64 + PCG32 XSH-RR keyed streams (src/effects/rng.rs:10-71,
// src/bake/random.rs:9-19) --------------------------------------------------------------------
DL_HD uint64_t splitmix64(uint64_t v) {
    v += 0x9e3779b97f4a7c15ull;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}
DL_HD uint64_t fold_seed(uint64_t acc, uint64_t part) { return splitmix64(acc ^ splitmix64(part)); }
constexpr uint64_t kSeedStart = 0x0b4ce5eed0000000ull;

struct Pcg {
    uint64_t state, inc;
    DL_HD uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
        uint32_t rot = (uint32_t)(old >> 59);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    DL_HD float next_f32() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
    // Jumps the state `delta` draws ahead in O(log delta) (Brown, "Random Number Generation with
    // Arbitrary Strides", 1994): the LCG step composed with itself by squaring.
    DL_HD void advance(uint64_t delta) {
        uint64_t mult = 6364136223846793005ull, plus = inc, acc_mult = 1, acc_plus = 0;
        while (delta) {
            if (delta & 1) {
                acc_mult *= mult;
                acc_plus = acc_plus * mult + plus;
            }
            plus = (mult + 1) * plus;
            mult *= mult;
            delta >>= 1;
        }
        state = acc_mult * state + acc_plus;
    }
};
DL_HD Pcg pcg_new(uint64_t seed, uint64_t stream) {
    Pcg r{0, (stream << 1) | 1};
    r.next_u32();
    r.state += seed;
    r.next_u32();
    return r;
}
DL_HD Pcg pcg_from_seed(uint64_t s) { return pcg_new(s, (s << 17) | (s >> 47)); }
// stream([a, b, c, ...]) for the key lengths the bake uses.
DL_HD Pcg stream4(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    return pcg_from_seed(fold_seed(fold_seed(fold_seed(fold_seed(kSeedStart, a), b), c), d));
}
DL_HD Pcg stream5(uint64_t a, uint64_t b, uint64_t c, uint64_t d, uint64_t e) {
    return pcg_from_seed(fold_seed(fold_seed(fold_seed(fold_seed(fold_seed(kSeedStart, a), b), c), d), e));
}
DL_HD Pcg stream6(uint64_t a, uint64_t b, uint64_t c, uint64_t d, uint64_t e, uint64_t f) {
    return pcg_from_seed(
        fold_seed(fold_seed(fold_seed(fold_seed(fold_seed(fold_seed(kSeedStart, a), b), c), d), e), f));
}
// random.rs:22-27
DL_HD f3 on_unit_sphere(Pcg &rng) {
    float z = rng.next_f32() * 2.0f - 1.0f;
    float angle = rng.next_f32() * kTau;
    float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
    float s, c;
    sincos_f(angle, s, c);
    return f3{r * c, r * s, z};
}

// ---- low-discrepancy points (src/bake/spread.rs) ----------------------------------------------
DL_HD uint32_t rev_bits(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __brev(v);
#else
    v = ((v >> 1) & 0x55555555u) | ((v & 0x55555555u) << 1);
    v = ((v >> 2) & 0x33333333u) | ((v & 0x33333333u) << 2);
    v = ((v >> 4) & 0x0F0F0F0Fu) | ((v & 0x0F0F0F0Fu) << 4);
    v = ((v >> 8) & 0x00FF00FFu) | ((v & 0x00FF00FFu) << 8);
    return (v >> 16) | (v << 16);
#endif
}
// The second coordinate of the (0, 2)-sequence (spread.rs:43-53): index bit k XORs in the
// direction number v_k, v_0 = 2^31 and v_(k+1) = v_k ^ (v_k >> 1), so v_k has bit 31 - j set
// exactly when j is a bit subset of k (Lucas). Bit 31 - j of the result is therefore the parity
// of the index bits k that are supersets of j: a superset-parity transform over the 32 bit
// positions (five shift-mask-xor steps) followed by a bit reversal, without a loop.
DL_HD uint32_t sobol2(uint32_t index) {
    uint32_t x = index;
    x ^= (x >> 1) & 0x55555555u;
    x ^= (x >> 2) & 0x33333333u;
    x ^= (x >> 4) & 0x0F0F0F0Fu;
    x ^= (x >> 8) & 0x00FF00FFu;
    x ^= (x >> 16) & 0x0000FFFFu;
    return rev_bits(x);
}
DL_HD float unit24(uint32_t bits) { return (float)(bits >> 8) / 16777216.0f; }
DL_HD f2 spread(uint32_t index, f2 off, bool rect) {
    float across = unit24(rev_bits(index));
    float down = rect ? unit24(sobol2(index)) : 0.0f;
    float a = across + off.x, d = down + off.y;
    return f2{a - floorf(a), d - floorf(d)};
}
// Shirley–Chiu concentric map (spread.rs:28-39).
DL_HD f2 concentric(f2 sq) {
    float px = sq.x * 2.0f - 1.0f, py = sq.y * 2.0f - 1.0f;
    if (px == 0.0f && py == 0.0f) return f2{0.0f, 0.0f};
    float radius, angle;
    if (fabsf(px) > fabsf(py)) {
        radius = px;
        angle = kFracPi4 * (py / px);
    } else {
        radius = py;
        angle = 2.0f * kFracPi4 - kFracPi4 * (px / py);
    }
    float s, c;
    sincos_f(angle, s, c);
    return f2{c * radius, s * radius};
}
// Malley's method (sky.rs:20-25), with the normal's orthonormal pair already computed.
DL_HD f3 cosine_direction_basis(f3 n, f3 side, f3 across, f2 sq) {
    f2 d = concentric(sq);
    float up = sqrtf(fmaxf(1.0f - (d.x * d.x + d.y * d.y), 0.0f));
    return normalize(add(add(scale(side, d.x), scale(across, d.y)), scale(n, up)));
}
DL_HD f3 cosine_direction(f3 n, f2 sq) {
    f3 side, across;
    ortho_pair(n, side, across);
    return cosine_direction_basis(n, side, across, sq);
}

// shadow_grid.rs:13-16
DL_HD uint32_t level_of(float fraction, uint32_t bits) {
    float max = (float)((1u << bits) - 1);
    return f2u8(roundf(clampf(fraction, 0.0f, 1.0f) * max));
}

}  // namespace dl
