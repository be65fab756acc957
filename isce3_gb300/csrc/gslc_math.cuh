// Host/device math for the SLC geocoder.
//
// Where the reference computes in FP32 (the biquintic DEM spline,
// cxx/isce3/core/Spline2dInterpolator.cpp:32-108) the device code uses
// round-to-nearest intrinsics so nvcc cannot contract or reorder: one ULP of
// DEM height moves the flattening phase by ~4e-3 rad at L-band, far above the
// 1e-4 rad parity tolerance.  FP64 geometry may contract to FMA; its
// differences stay ~1e-16 relative.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define GSLC_HD __host__ __device__ __forceinline__
#define GSLC_HD_COLD __host__ __device__ __noinline__ inline
#else
#define GSLC_HD inline
#define GSLC_HD_COLD inline
#endif

namespace gslc {

// ---- exact-order FP32 / FP64 primitives (device: _rn intrinsics) ----------
#if defined(__CUDA_ARCH__)
GSLC_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
GSLC_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
GSLC_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
GSLC_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
GSLC_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
GSLC_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
GSLC_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
GSLC_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
#else
GSLC_HD float fadd(float a, float b) { return a + b; }
GSLC_HD float fsub(float a, float b) { return a - b; }
GSLC_HD float fmul(float a, float b) { return a * b; }
GSLC_HD float fdiv(float a, float b) { return a / b; }
GSLC_HD double dadd(double a, double b) { return a + b; }
GSLC_HD double dsub(double a, double b) { return a - b; }
GSLC_HD double dmul(double a, double b) { return a * b; }
GSLC_HD double ddiv(double a, double b) { return a / b; }
#endif

constexpr double PI = 3.14159265358979323846;
constexpr double WGS84_A = 6378137.0;                 // core/Constants.h:41
constexpr double WGS84_E2 = 0.006694379990141317;     // core/Constants.h:44
constexpr int SINC_HALF = 4, SINC_LEN = 8, SINC_ONE = 9, SINC_SUB = 8192;  // core/Constants.h:32-35

struct V3 { double x, y, z; };
GSLC_HD V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
GSLC_HD double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GSLC_HD V3 vcross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
GSLC_HD double vnorm(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// Bits of a double.  For |x| < c with c > 0, comparing the magnitude bits
// (sign cleared) as unsigned integers gives the same answer as the FP64
// compare, NaN included (its magnitude bits exceed every finite c's); the
// Newton loop uses it to keep its tests off the FP64 pipe.
GSLC_HD uint64_t dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof(u));
    return u;
#endif
}
constexpr uint64_t DMAG = 0x7fffffffffffffffull;
constexpr uint64_t DBITS_HALF = 0x3fe0000000000000ull;        // 0.5
constexpr uint64_t DBITS_MINUS_HALF = 0xbfe0000000000000ull;  // -0.5
constexpr uint64_t DBITS_0P1 = 0x3fb999999999999aull;         // 0.1

// Order key of a double: for finite x, y (and -0.0 == +0.0), x <= y exactly
// when dkey(x) <= dkey(y) as signed integers.  A NaN's key lies above every
// finite key (positive sign) or below it (negative sign), so a two-sided
// test lo <= x <= hi is false for it, as the FP64 test is.  Range tests use
// it to stay off the FP64 pipe.
GSLC_HD int64_t dkey(double x) {
    const int64_t b = (int64_t)dbits(x);
    return b < 0 ? -(b & (int64_t)DMAG) : b;
}
constexpr int64_t DKEY_INF = 0x7ff0000000000000ll;   // dkey(+inf); above it: NaN

// Integer part and fraction of x from its bits, both exact, off the FP64
// pipe: for x in [1, 2^31) returns trunc(x) and sets frac64 to
// (x - trunc(x)) * 2^64 (the bits of x below the binary point, moved to the
// top of the word); for x in [0, 1) returns 0; for x >= 2^31, infinite, NaN
// or with the sign bit set returns INT32_MAX.  frac64 is 0 in the last two
// cases.
GSLC_HD int32_t split_bits(double x, uint64_t& frac64) {
    const uint64_t b = dbits(x);
    const int e = (int)(b >> 52) - 1023;
    frac64 = 0;
    if (e < 0) return 0;
    if (e > 30) return 0x7fffffff;
    const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
    frac64 = m << (12 + e);
    return (int32_t)(m >> (52 - e));
}

// frac64 * 2^-64 rounded to the nearest float, ties to even: the float of
// a fraction split_bits formed, as converting the exact double would give.
GSLC_HD float fixed64_to_float(uint64_t f) {
    if (f == 0) return 0.0f;
#if defined(__CUDA_ARCH__)
    const int lz = __clzll((long long)f);
#else
    const int lz = __builtin_clzll(f);
#endif
    const uint64_t n = f << lz;                     // leading one at bit 63
    uint32_t mant = (uint32_t)(n >> 40);            // 24 bits, leading one at bit 23
    const uint64_t rest = n & 0xffffffffffull;      // the 40 bits below
    const uint64_t half = 1ull << 39;
    if (rest > half || (rest == half && (mant & 1u))) ++mant;
    uint32_t expo = 126u - (uint32_t)lz;            // n * 2^(-64-lz) = (mant / 2^23) * 2^(-1-lz)
    if (mant == (1u << 24)) {
        mant >>= 1;
        ++expo;
    }
    const uint32_t u = (expo << 23) | (mant & 0x7fffffu);
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float r;
    memcpy(&r, &u, sizeof(r));
    return r;
#endif
}

// (float)n for |n| < 2^22: 1.5 * 2^23 + n is exact in float, so its bits
// are those of 1.5 * 2^23 plus n; an integer add and an FP32 subtraction,
// off the conversion unit.
GSLC_HD float small_int_to_float(int32_t n) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(0x4B400000u + (uint32_t)n) - 12582912.0f;
#else
    return (float)n;
#endif
}

// (int)floor(x): the integer part from the bits where x is in [0, 2^31)
// (split_bits, off the FP64 pipe), the FP64 floor elsewhere.
GSLC_HD int floor_int(double x) {
    uint64_t f;
    const int32_t i = split_bits(x, f);
    return i != 0x7fffffff ? (int)i : (int)floor(x);
}

// ---- LUT2d (core/LUT2d.{h,cpp}) ------------------------------------------
struct Lut {
    int32_t have_data, bounds_error, method, nx, ny, _pad;
    double x0, y0, dx, dy, ref_value;
    double inv_dx, inv_dy;      // 1/dx, 1/dy
    // contains(y, x) (core/LUT2d.h:84-95) as order keys: it holds exactly
    // where kx_lo <= dkey(x) <= kx_hi and ky_lo <= dkey(y) <= ky_hi (the
    // host finds the bounds with the reference's expression)
    int64_t kx_lo, kx_hi, ky_lo, ky_hi;
    const double* data;
    const double* sinc;         // method 0: the sinc kernel table in double, [SINC_SUB][SINC_LEN]
};

// Host side (launch preparation): the key intervals of Lut and GeoParams.
// The double whose order key (dkey) is k, for the keys of finite doubles.
inline double key_double(int64_t k) {
    const uint64_t b = k >= 0 ? (uint64_t)k : ((uint64_t)(-k) | 0x8000000000000000ull);
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
}

// Order keys [lo, hi] of the finite x where g(x) >= 0.0 and g(x) <= top hold
// together, for g monotone in x (non-decreasing when up, else
// non-increasing) and never NaN there: each test is monotone in x, so its
// boundary is found by bisection over the keys, evaluating g as the
// reference writes it.  Empty: lo > hi.
template <class G>
inline void key_interval(G g, bool up, double top, int64_t& lo, int64_t& hi) {
    const int64_t kmax = dkey(1.7976931348623157e308);   // the largest finite double
    // first key in [-kmax, kmax] where pred holds (pred false, then true), kmax + 1 if none
    auto first = [&](auto pred) {
        int64_t a = -kmax, b = kmax + 1;
        while (a < b) {
            const int64_t m = a + (int64_t)(((uint64_t)b - (uint64_t)a) / 2);
            if (pred(key_double(m))) b = m;
            else a = m + 1;
        }
        return a;
    };
    if (up) {
        lo = first([&](double x) { return g(x) >= 0.0; });
        hi = first([&](double x) { return !(g(x) <= top); }) - 1;
    } else {
        lo = first([&](double x) { return g(x) <= top; });
        hi = first([&](double x) { return !(g(x) >= 0.0); }) - 1;
    }
}

// The keys of one axis of LUT2d::contains (core/LUT2d.h:84-95):
// (x - x0) / dx in [0, n - 1].  A spacing of zero or NaN, or an origin that
// is not finite, contains nothing; an infinite spacing contains every
// finite x (the quotient is zero) when n >= 1.
inline void lut_axis_keys(double x0, double dx, int n, int64_t& lo, int64_t& hi) {
    const int64_t kmax = dkey(1.7976931348623157e308);   // the largest finite double
    lo = 1;
    hi = 0;
    if (!isfinite(x0) || !(dx != 0.0)) return;
    if (isinf(dx)) {
        if (n >= 1) { lo = -kmax; hi = kmax; }
        return;
    }
    key_interval([&](double x) { return (x - x0) / dx; }, dx > 0, n - 1.0, lo, hi);
}

// core/LUT2d.h:84-95: (x - xStart) / dx in [0, width - 1] and likewise in
// y, which is monotone in x (in y), so it holds on an interval of each; the
// test compares order keys with the interval's ends (Lut::kx_lo ...), the
// same decision as the reference's for every x and y, off the FP64 pipe.
GSLC_HD bool lut_contains(const Lut& l, double y, double x) {
    if (!l.have_data) return true;
    const int64_t kx = dkey(x), ky = dkey(y);
    return kx >= l.kx_lo && kx <= l.kx_hi && ky >= l.ky_lo && ky <= l.ky_hi;
}

// (float)x from the bits with integer operations (off the FP64 pipe),
// rounded to nearest even, where x is zero or rounds to a normal float;
// other values (float subnormals, overflow, infinities, NaN) take the
// conversion instruction.
GSLC_HD float dbl_to_float(double x) {
    const uint64_t b = dbits(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;   // the float's biased exponent
    uint32_t u;
    if ((b & DMAG) == 0) {
        u = sign;
    } else if (e < 1 || e > 254) {
        return (float)x;
    } else {
        const uint64_t m = b & 0xfffffffffffffull;
        u = ((uint32_t)e << 23) | (uint32_t)(m >> 29);
        const uint64_t rest = m & 0x1fffffffull, half = 1ull << 28;
        if (rest > half || (rest == half && (u & 1u))) ++u;   // a carry into the exponent rounds up correctly
        u |= sign;
    }
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float r;
    memcpy(&r, &u, sizeof(r));
    return r;
#endif
}

// a load through a pointer that may address shared memory
template <typename T>
GSLC_HD T ld_gen(const T* p) {
    return *p;
}

template <typename T>
GSLC_HD T ld_ro(const T* p) {
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

// ---- LUT2d's other interpolators, FP64 in the reference's operation order,
// at table coordinates already clamped to the table (LUT2d.cpp:151-152) ----
GSLC_HD double lut_at(const Lut& l, int r, int c) {
    r = r < 0 ? 0 : (r > l.ny - 1 ? l.ny - 1 : r);
    c = c < 0 ? 0 : (c > l.nx - 1 ? l.nx - 1 : c);
    return ld_ro(l.data + (long)r * l.nx + c);
}

// core/BicubicInterpolator.cpp:37-42 (cubicInterpolate, T = double)
GSLC_HD double lut_cubic(double p0, double p1, double p2, double p3, double t) {
    const double tc = dsub(1.0, t);
    const double inner = dadd(dsub(p2, dmul(p0, dmul(tc, tc))),
                              dmul(dsub(dmul(p2, dadd(dmul(tc, 3.0), 1.0)), dmul(p3, tc)), t));
    const double tail = dmul(p1, dadd(dmul(dmul(t, t), dsub(dmul(t, 3.0), 5.0)), 2.0));
    return ddiv(dadd(dmul(t, inner), tail), 2.0);
}

// core/BicubicInterpolator.cpp:47-64: rows y0-1..y0+2, columns x0-1..x0+2.
// The reference reads that neighbourhood unchecked, which at a table's edge
// rows and columns falls outside the table; those reads are clamped here.
GSLC_HD double lut_bicubic(const Lut& l, double xi, double yi) {
    const int x0 = (int)floor(xi), y0 = (int)floor(yi);
    const double fx = dsub(xi, (double)x0), fy = dsub(yi, (double)y0);
    double v[4];
    for (int i = -1; i < 3; ++i)
        v[i + 1] = lut_cubic(lut_at(l, y0 + i, x0 - 1), lut_at(l, y0 + i, x0), lut_at(l, y0 + i, x0 + 1),
                             lut_at(l, y0 + i, x0 + 2), fx);
    return lut_cubic(v[0], v[1], v[2], v[3], fy);
}

// core/Spline2dInterpolator.cpp:89-108 (_initSpline, U = double, n = 6)
GSLC_HD void lut_init_spline6(const double Y[6], double R[6]) {
    double Q[6];
    Q[0] = 0.0;
    R[0] = 0.0;
    for (int i = 1; i < 5; ++i) {
        const double p = ddiv(1.0, dadd(dmul(0.5, Q[i - 1]), 2.0));
        Q[i] = dmul(-0.5, p);
        R[i] = dmul(dsub(dmul(3.0, dadd(dsub(Y[i + 1], dmul(2.0, Y[i])), Y[i - 1])), dmul(0.5, R[i - 1])), p);
    }
    R[5] = 0.0;
    for (int i = 4; i > 0; --i) R[i] = dadd(dmul(Q[i], R[i + 1]), R[i]);
}

// core/Spline2dInterpolator.cpp:69-87 (_spline) on the branch x in [2, 3)
// that LUT2d's clamped coordinates always take (x - j0 = 2 + frac)
GSLC_HD double lut_spline6_at(double x, const double Y[6], const double R[6]) {
    const int j = (int)floor(x);
    const double xx = dsub(x, (double)j);
    const double t0 = dsub(dsub(dsub(Y[j], Y[j - 1]), ddiv(R[j - 1], 3.0)), ddiv(R[j], 6.0));
    const double t1 = dmul(xx, dadd(ddiv(R[j - 1], 2.0), dmul(xx, ddiv(dsub(R[j], R[j - 1]), 6.0))));
    return dadd(Y[j - 1], dmul(xx, dadd(t0, t1)));
}

// core/Spline2dInterpolator.cpp:32-67 (interp_impl, order 6): window rows and
// columns clamped to [0, n - 2], read at index + 1
GSLC_HD double lut_biquintic(const Lut& l, double xi, double yi) {
    const int i0 = (int)yi - 2, j0 = (int)xi - 2;
    double A[6], R[6], HC[6];
    for (int i = 0; i < 6; ++i) {
        int indi = i0 + i;
        indi = (indi < 0 ? 0 : (indi > l.ny - 2 ? l.ny - 2 : indi)) + 1;
        for (int j = 0; j < 6; ++j) {
            int indj = j0 + j;
            indj = (indj < 0 ? 0 : (indj > l.nx - 2 ? l.nx - 2 : indj)) + 1;
            A[j] = ld_ro(l.data + (long)indi * l.nx + indj);
        }
        lut_init_spline6(A, R);
        HC[i] = lut_spline6_at(dsub(xi, (double)j0), A, R);
    }
    lut_init_spline6(HC, R);
    return lut_spline6_at(dsub(yi, (double)i0), HC, R);
}

// core/Sinc2dInterpolator.cpp:45-96 (U = double): 8 x 8 taps, 0 within 3-4
// samples of the table's edges
GSLC_HD double lut_sinc(const Lut& l, double xi, double yi) {
    const int ix = (int)floor(xi), iy = (int)floor(yi);
    const double fx = dsub(xi, (double)ix), fy = dsub(yi, (double)iy);
    if (ix < SINC_HALF - 1 || ix > l.nx - SINC_HALF - 1) return 0.0;
    if (iy < SINC_HALF - 1 || iy > l.ny - SINC_HALF - 1) return 0.0;
    const int xx = ix + SINC_HALF, yy = iy + SINC_HALF;
    int fxi = (int)dmul(fx, (double)SINC_SUB), fyi = (int)dmul(fy, (double)SINC_SUB);
    fxi = fxi < 0 ? 0 : (fxi > SINC_SUB - 1 ? SINC_SUB - 1 : fxi);
    fyi = fyi < 0 ? 0 : (fyi > SINC_SUB - 1 ? SINC_SUB - 1 : fyi);
    double ret = 0.0;
    for (int i = 0; i < SINC_LEN; ++i)
        for (int j = 0; j < SINC_LEN; ++j)
            ret = dadd(ret, dmul(dmul(ld_ro(l.data + (long)(yy - i) * l.nx + (xx - j)),
                                      ld_ro(l.sinc + fyi * SINC_LEN + i)),
                                 ld_ro(l.sinc + fxi * SINC_LEN + j)));
    return ret;
}

// methods 0 (sinc), 2 (bicubic) and 4 (biquintic) at clamped table
// coordinates; out of line, so that the geocode kernels' register allocation
// does not carry these rarely taken paths
GSLC_HD_COLD double lut_interp_other(const Lut& l, double xi, double yi) {
    if (l.method == 2) return lut_bicubic(l, xi, yi);
    if (l.method == 4) return lut_biquintic(l, xi, yi);
    return lut_sinc(l, xi, yi);
}

// core/LUT2d.cpp:124-158 with core/BilinearInterpolator.cpp:12-49 or
// core/NearestNeighborInterpolator.cpp:12-22.  The bilinear divisions by
// (x2-x1)*(y2-y1) == 1 are exact and omitted.
GSLC_HD double lut_eval(const Lut& l, double y, double x) {
    if (!l.have_data) return l.ref_value;
    double xi = (x - l.x0) * l.inv_dx;
    double yi = (y - l.y0) * l.inv_dy;
    xi = fmin(fmax(xi, 0.0), l.nx - 1.0);
    yi = fmin(fmax(yi, 0.0), l.ny - 1.0);
    if (l.method != 1 && l.method != 3) return lut_interp_other(l, xi, yi);
    if (l.method == 3) {
        long r = (long)round(yi), c = (long)round(xi);
        return ld_ro(l.data + r * l.nx + c);
    }
    const int x1 = (int)floor(xi), x2 = (int)ceil(xi);
    const int y1 = (int)floor(yi), y2 = (int)ceil(yi);
    const double q11 = ld_ro(l.data + (long)y1 * l.nx + x1), q12 = ld_ro(l.data + (long)y2 * l.nx + x1);
    const double q21 = ld_ro(l.data + (long)y1 * l.nx + x2), q22 = ld_ro(l.data + (long)y2 * l.nx + x2);
    if (y1 == y2 && x1 == x2) return q11;
    if (y1 == y2) return (x2 - xi) * q11 + (xi - x1) * q21;
    if (x1 == x2) return (y2 - yi) * q11 + (yi - y1) * q12;
    return q11 * ((x2 - xi) * (y2 - yi)) + q21 * ((xi - x1) * (y2 - yi)) +
           q12 * ((x2 - xi) * (yi - y1)) + q22 * ((xi - x1) * (yi - y1));
}

// ---- Poly2d (core/Poly2d.cpp:8-24) ----------------------------------------
constexpr int POLY_MAX = 64;
struct Poly {
    int32_t x_order, y_order;
    double x_mean, y_mean, x_norm, y_norm;
    double inv_x_norm, inv_y_norm;
    double c[POLY_MAX];
};

// The LUT's value in FP32 for values that only set float phases (the
// native Doppler of the sinc chip, whose phasors are float angles): the
// bilinear at table coordinates formed in FP32, relative error ~1e-7 of
// the value; the other methods in FP64, whose rounding picks the cell.
GSLC_HD float lut_bilinear_f32(const Lut& l, float xi, float yi);

// lut_contains(l, y, x), and where it holds v, the value in FP32 (above)
GSLC_HD bool lut_contains_eval_f32(const Lut& l, double y, double x, float& v) {
    if (!l.have_data) {
        v = (float)l.ref_value;
        return true;
    }
    if (!lut_contains(l, y, x)) return false;
    v = l.method != 1 ? (float)lut_eval(l, y, x)
                      : lut_bilinear_f32(l, (float)((x - l.x0) * l.inv_dx), (float)((y - l.y0) * l.inv_dy));
    return true;
}

// the bilinear (BilinearInterpolator.cpp:12-49) at table coordinates (xi, yi), in FP32
GSLC_HD float lut_bilinear_f32(const Lut& l, float xi, float yi) {
    xi = fminf(fmaxf(xi, 0.f), (float)(l.nx - 1));
    yi = fminf(fmaxf(yi, 0.f), (float)(l.ny - 1));
    const int x1 = (int)floorf(xi), x2 = (int)ceilf(xi);
    const int y1 = (int)floorf(yi), y2 = (int)ceilf(yi);
    const float q11 = dbl_to_float(ld_ro(l.data + (long)y1 * l.nx + x1));
    const float q12 = dbl_to_float(ld_ro(l.data + (long)y2 * l.nx + x1));
    const float q21 = dbl_to_float(ld_ro(l.data + (long)y1 * l.nx + x2));
    const float q22 = dbl_to_float(ld_ro(l.data + (long)y2 * l.nx + x2));
    const float wx2 = (float)x2 - xi, wx1 = xi - (float)x1, wy2 = (float)y2 - yi, wy1 = yi - (float)y1;
    if (y1 == y2 && x1 == x2) return q11;
    if (y1 == y2) return wx2 * q11 + wx1 * q21;
    if (x1 == x2) return wy2 * q11 + wy1 * q12;
    return q11 * (wx2 * wy2) + q21 * (wx1 * wy2) + q12 * (wx2 * wy1) + q22 * (wx1 * wy1);
}

// core/Poly2d.cpp:8-24: the sum of c[i][j] xval^j yval^i with
// xval = (x - xMean) / xNorm and yval likewise, here normalised with
// reciprocals and summed in nested Horner form, one FMA per coefficient
// (the term-by-term sum formed every power and product: 19 FP64
// instructions per pixel for the frame's two carriers against 4).  The
// rounding differs from the reference's by a few ulps of its largest term;
// it serves the reramp's FP64 phase, and the deramp, whose float phase must
// match the reference's, uses poly_eval_exact.
GSLC_HD double poly_eval(const Poly& p, double y, double x) {
    const double xval = p.x_order > 0 ? (x - p.x_mean) * p.inv_x_norm : 0.0;
    const double yval = p.y_order > 0 ? (y - p.y_mean) * p.inv_y_norm : 0.0;
    const int nx = p.x_order + 1;
    double val = 0.0;
    for (int i = p.y_order; i >= 0; --i) {
        const double* c = p.c + i * nx;
        double row = c[p.x_order];
        for (int j = p.x_order - 1; j >= 0; --j) row = fma(row, xval, c[j]);
        val = i == p.y_order ? row : fma(val, yval, row);
    }
    return val;
}

// Exact-order forms (no contraction, divisions as the reference writes
// them): the deramp rounds the carrier phase to float, so an ulp of FP64
// difference there can move the float phase by one float ulp.
// core/LUT2d.cpp:124-158 + core/BilinearInterpolator.cpp:12-49 (den == 1).
GSLC_HD double lut_eval_exact(const Lut& l, double y, double x) {
    if (!l.have_data) return l.ref_value;
    double xi = ddiv(dsub(x, l.x0), l.dx);
    double yi = ddiv(dsub(y, l.y0), l.dy);
    xi = fmin(fmax(xi, 0.0), l.nx - 1.0);
    yi = fmin(fmax(yi, 0.0), l.ny - 1.0);
    if (l.method != 1 && l.method != 3) return lut_interp_other(l, xi, yi);
    if (l.method == 3) {
        long r = (long)round(yi), c = (long)round(xi);
        return ld_ro(l.data + r * l.nx + c);
    }
    const int x1 = (int)floor(xi), x2 = (int)ceil(xi);
    const int y1 = (int)floor(yi), y2 = (int)ceil(yi);
    const double q11 = ld_ro(l.data + (long)y1 * l.nx + x1), q12 = ld_ro(l.data + (long)y2 * l.nx + x1);
    const double q21 = ld_ro(l.data + (long)y1 * l.nx + x2), q22 = ld_ro(l.data + (long)y2 * l.nx + x2);
    if (y1 == y2 && x1 == x2) return q11;
    if (y1 == y2) return dadd(dmul(dsub(x2, xi), q11), dmul(dsub(xi, x1), q21));
    if (x1 == x2) return dadd(dmul(dsub(y2, yi), q11), dmul(dsub(yi, y1), q12));
    double v = dmul(q11, dmul(dsub(x2, xi), dsub(y2, yi)));
    v = dadd(v, dmul(q21, dmul(dsub(xi, x1), dsub(y2, yi))));
    v = dadd(v, dmul(q12, dmul(dsub(x2, xi), dsub(yi, y1))));
    return dadd(v, dmul(q22, dmul(dsub(xi, x1), dsub(yi, y1))));
}

// core/Poly2d.cpp:8-24 with yval = (y - y_mean) / y_norm given
GSLC_HD double poly_eval_exact(const Poly& p, double yval, double x) {
    const double xval = p.x_order > 0 ? ddiv(dsub(x, p.x_mean), p.x_norm) : 0.0;  // unused at order 0
    double scaley = 1., val = 0.;
    for (int i = 0; i <= p.y_order; i++, scaley = dmul(scaley, yval)) {
        double scalex = 1.;
        for (int j = 0; j <= p.x_order; j++, scalex = dmul(scalex, xval))
            val = dadd(val, dmul(dmul(scalex, scaley), p.c[i * (p.x_order + 1) + j]));
    }
    return val;
}

struct AzRg {
    int32_t kind;      // 0 LUT2d, 1 Poly2d
    int32_t is_zero;   // evaluates to exactly 0 everywhere (default object)
    Lut lut;
    Poly poly;
};

GSLC_HD double azrg_eval(const AzRg& f, double y, double x) {
    if (f.is_zero) return 0.0;
    return f.kind == 1 ? poly_eval(f.poly, y, x) : lut_eval(f.lut, y, x);
}

// ---- Ellipsoid (core/Ellipsoid.h:117-120, 177-190) -------------------------
GSLC_HD V3 lonlat_to_xyz(double a, double e2, double lon, double lat, double h) {
    double slat, clat, slon, clon;
#if defined(__CUDA_ARCH__)
    sincos(lat, &slat, &clat);
    sincos(lon, &slon, &clon);
#else
    slat = sin(lat); clat = cos(lat); slon = sin(lon); clon = cos(lon);
#endif
    const double re = a / sqrt(1.0 - e2 * (slat * slat));
    return {(re + h) * clat * clon, (re + h) * clat * slon, ((re * (1.0 - e2)) + h) * slat};
}

// lonLatToXyz from precomputed sines and cosines
GSLC_HD V3 lonlat_to_xyz_sc(double a, double e2, double slon, double clon, double slat, double clat, double h) {
    const double re = a / sqrt(1.0 - e2 * (slat * slat));
    return {(re + h) * clat * clon, (re + h) * clat * slon, ((re * (1.0 - e2)) + h) * slat};
}

// ---- Projections (core/Projections.{h,cpp}) -------------------------------
struct Utm {
    int32_t isnorth, _pad;
    double lon0, Qn, Zb;
    double slon0, clon0;        // sin/cos of the central meridian
    double cgb[6], cbg[6], utg[6], gtu[6];
};

// core/Projections.cpp:33-42 (real Clenshaw summation)
GSLC_HD double clens(const double* a, double real) {
    const double cr = cos(real);
    double hr2 = 0., hr1 = a[5], hr = 0.;
    for (int k = 4; k >= 0; --k) {
        hr = -hr2 + (2. * hr1 * cr) + a[k];
        hr2 = hr1;
        hr1 = hr;
    }
    return sin(real) * hr;
}

// core/Projections.cpp:54-74 (complex Clenshaw summation).  The row/column
// factors sin/cos(real) and sinh/cosh(imag) are evaluated once.
GSLC_HD void clenS(const double* a, double sr, double cr, double shi, double chi, double& R, double& I) {
    double hr2 = 0., hi2 = 0., hi1 = 0., hr1 = a[5], hr = 0., hi = 0.;
    const double rr = 2. * cr * chi, ii = -2. * sr * shi;
    for (int k = 4; k >= 0; --k) {
        hr = -hr2 + (hr1 * rr) - (hi1 * ii) + a[k];
        hi = -hi2 + (hr1 * ii) + (hi1 * rr);
        hr2 = hr1; hi2 = hi1; hr1 = hr; hi1 = hi;
    }
    R = (sr * chi * hr) - (cr * shi * hi);
    I = (sr * chi * hi) + (cr * shi * hr);
}

// core/Projections.cpp:200-232; returns false where the reference throws.
GSLC_HD bool utm_inverse(const Utm& u, double x, double y, double& lon, double& lat) {
    double Cn = (y - (u.isnorth ? 0. : 10000000.)) / WGS84_A;
    double Ce = (x - 500000.) / WGS84_A;
    Cn = (Cn - u.Zb) / u.Qn;
    Ce /= u.Qn;
    if (!(fabs(Ce) <= 2.623395162778)) return false;
    double sr, cr;
#if defined(__CUDA_ARCH__)
    sincos(2 * Cn, &sr, &cr);
#else
    sr = sin(2 * Cn); cr = cos(2 * Cn);
#endif
    const double shi = sinh(2 * Ce), chi = cosh(2 * Ce);
    double dCn, dCe;
    clenS(u.utg, sr, cr, shi, chi, dCn, dCe);
    Cn += dCn;
    Ce = atan(sinh(Ce + dCe));
    double sinCe, cosCe, sinCn, cosCn;
#if defined(__CUDA_ARCH__)
    sincos(Ce, &sinCe, &cosCe);
    sincos(Cn, &sinCn, &cosCn);
#else
    sinCe = sin(Ce); cosCe = cos(Ce); sinCn = sin(Cn); cosCn = cos(Cn);
#endif
    Ce = atan2(sinCe, cosCe * cosCn);
    Cn = atan2(sinCn * cosCe, hypot(sinCe, cosCe * cosCn));
    lon = Ce + u.lon0;
    lat = clens(u.cgb, 2 * Cn) + Cn;
    return true;
}

// The UTM inverse split by what it depends on.  Easting-only terms
// (Projections.cpp:203-210): normalised easting and sinh/cosh of twice it.
struct UtmCol { double Ce, shi, chi; int ok; };
GSLC_HD UtmCol utm_inverse_col(const Utm& u, double x) {
    UtmCol c;
    c.Ce = ((x - 500000.) / WGS84_A) / u.Qn;
    c.ok = fabs(c.Ce) <= 2.623395162778;
    c.shi = sinh(2 * c.Ce);
    c.chi = cosh(2 * c.Ce);
    return c;
}
// Northing-only terms: normalised northing and sin/cos of twice it.
struct UtmRow { double Cn, sr, cr; };
GSLC_HD UtmRow utm_inverse_row(const Utm& u, double y) {
    UtmRow r;
    r.Cn = ((y - (u.isnorth ? 0. : 10000000.)) / WGS84_A - u.Zb) / u.Qn;
#if defined(__CUDA_ARCH__)
    sincos(2 * r.Cn, &r.sr, &r.cr);
#else
    r.sr = sin(2 * r.Cn); r.cr = cos(2 * r.Cn);
#endif
    return r;
}

// Per-pixel remainder of the UTM inverse, with the transcendentals the
// reference chains replaced by identities:
//   atan(sinh x): sin = tanh x, cos = sech x (Gudermannian), from expm1;
//   sin/cos of the Gaussian latitude are the atan2 operands (B^2 + H^2 = 1);
//   sin/cos of the latitude rotate those by the small Clenshaw correction d
//   (|d| < 3.4e-3, series to d^6: error < 1e-20);
//   sin/cos of the longitude rotate (sinCe, A)/H by the central meridian.
// Returns lon, lat (rad) and their sines and cosines.
struct LonLatSC { double lon, lat, slon, clon, slat, clat; };
GSLC_HD LonLatSC utm_inverse_px(const Utm& u, const UtmRow& r, const UtmCol& c) {
    double dCn, dCe;
    clenS(u.utg, r.sr, r.cr, c.shi, c.chi, dCn, dCe);
    const double Cn1 = r.Cn + dCn;
    const double xg = c.Ce + dCe;
    const double em = expm1(xg);
    const double num = em * (2.0 + em);            // e^(2x) - 1
    const double q = 1.0 / (num + 2.0);            // 1 / (e^(2x) + 1)
    const double sinCe = num * q;                  // tanh x
    const double cosCe = (2.0 + 2.0 * em) * q;     // sech x
    double sinCn, cosCn;
#if defined(__CUDA_ARCH__)
    sincos(Cn1, &sinCn, &cosCn);
#else
    sinCn = sin(Cn1); cosCn = cos(Cn1);
#endif
    const double A = cosCe * cosCn;
    const double H = hypot(sinCe, A);
    const double B = sinCn * cosCe;
    LonLatSC o;
    o.lon = atan2(sinCe, A) + u.lon0;
    const double Cg = atan2(B, H);
    // clens(cgb, 2 Cg) (Projections.cpp:33-42) with sin/cos(2 Cg) = (2BH, H^2 - B^2)
    const double s2 = 2.0 * B * H, tc = 2.0 * ((H - B) * (H + B));
    double hr2 = 0., hr1 = u.cgb[5], hr = 0.;
    for (int k = 4; k >= 0; --k) {
        hr = -hr2 + hr1 * tc + u.cgb[k];
        hr2 = hr1;
        hr1 = hr;
    }
    const double d = s2 * hr;
    o.lat = Cg + d;
    const double d2 = d * d;
    const double sd = d * (1.0 - d2 * (1.0 / 6.0 - d2 * (1.0 / 120.0)));
    const double cd = 1.0 - d2 * (0.5 - d2 * (1.0 / 24.0 - d2 * (1.0 / 720.0)));
    o.slat = B * cd + H * sd;
    o.clat = H * cd - B * sd;
    const double iH = 1.0 / H;
    const double sl = sinCe * iH, cl = A * iH;
    o.slon = sl * u.clon0 + cl * u.slon0;
    o.clon = cl * u.clon0 - sl * u.slon0;
    return o;
}

// core/Projections.cpp:172-198
GSLC_HD bool utm_forward(const Utm& u, double lon, double lat, double& x, double& y) {
    const double gauss = clens(u.cbg, 2. * lat) + lat;
    const double lam = lon - u.lon0;
    double Cn = atan2(sin(gauss), cos(lam) * cos(gauss));
    double Ce = atan2(sin(lam) * cos(gauss), hypot(sin(gauss), cos(gauss) * cos(lam)));
    Ce = asinh(tan(Ce));
    double dCn, dCe;
    clenS(u.gtu, sin(2 * Cn), cos(2 * Cn), sinh(2 * Ce), cosh(2 * Ce), dCn, dCe);
    Cn += dCn;
    Ce += dCe;
    if (!(fabs(Ce) <= 2.623395162778)) return false;
    x = (u.Qn * Ce * WGS84_A) + 500000.;
    y = (((u.Qn * Cn) + u.Zb) * WGS84_A) + (u.isnorth ? 0. : 10000000.);
    return true;
}

// ---- Orbit as per-interval polynomials -------------------------------------
// The 4-point Hermite interpolant of core/detail/InterpolateOrbit.icc:10-109
// is, on each state-vector interval, one degree-7 polynomial in
// u = (t - t_idx)/spacing - 1.5; velocity is its derivative.  The host
// expands it once per interval (gslc_capi.cu) around P_ref = P_{idx+1}.
constexpr int ORB_STRIDE = 48;   // pref[3], a[3][8], b[3][7] (b = d/dt coefficients)

// Newton tables per state-vector interval ("segment" j = 0..n-2, the time
// span [t_j, t_j+1]).  Segment j uses the Hermite piece
// idx = clamp(j - 1, 0, n - 4), re-expanded in w = u - (j - idx - 1) so that
// w lies in [-0.5, 0.5] on the segment (w = u for interior segments).  With
// D = xyz - P_ref, the zero-Doppler residual of geo2rdr is
//   (xyz - pos(w)) . vel(w) = D . vel(w) - H(w),   H(w) = a(w) . vel(w),
// and the Newton step divides by -|vel(w)|^2 = -1 / G(w).  H is a degree-13
// polynomial (truncated where its tail is below 1e-9 m^2/s), G a truncated
// power series of 1/|vel|^2 accurate to about one ulp on the segment.
constexpr int SEG_NH = 14, SEG_NG = 13;
constexpr int SEG_STRIDE = 76;   // pref[3], a[3][8], b[3][7], h[14], g[13], t
constexpr int SEG_A = 3, SEG_B = 27, SEG_H = 48, SEG_G = 62;
// t: the segment's start time t0 + j * spacing, rounded once (an FMA), as
// the Newton forms it; read where the iterate enters a segment instead of
// converting the index (two FP64-pipe conversions and two FMAs saved)
constexpr int SEG_T = 75;
// The same segment tables as float pairs (hi, lo) for the float-float Newton.
constexpr int SEGFF_STRIDE = 72;   // float2: b[3][7], h[14], g[13], a[3][8]
constexpr int SEGFF_B = 0, SEGFF_H = 21, SEGFF_G = 35, SEGFF_A = 48;

struct Orbit {
    double t0, spacing, inv_spacing, t_end;
    int32_t n, n_pieces;
    const double* coef;          // n_pieces * ORB_STRIDE
    const double* seg;           // (n - 1) * SEG_STRIDE
    const float2* seg_ff;        // (n - 1) * SEGFF_STRIDE
    int32_t seg_nh, seg_ng;      // highest H and G degree used over all segments
    int32_t seg_div;             // 1: G did not converge, divide by -|vel|^2 instead
    int32_t seg_a7;              // 1: the position's degree-7 term matters (else degree 6)
    int32_t legendre;            // 1: Legendre interpolation; coef holds the state vectors
                                 // (positions 3n, then velocities 3n) and seg, seg_ff are unused
    int32_t seg_r6;              // 1: the residual's degree-6 term is kept (else degree 5)
    // the degree-6 term's step over |w| <= 1/2, max over segments: up to
    // |D| seg_b6 + seg_h6 seconds for |D| = |xyz - P_ref| (seconds per metre, seconds)
    double seg_b6, seg_h6;
};

// Orbit table layout in doubles: the pieces, then the segments (16-byte
// aligned), then the segments' float pairs (SEG_STRIDE is even, so aligned).
constexpr size_t orbit_seg_offset(int n) { return ((size_t)(n - 3) * ORB_STRIDE + 1) & ~(size_t)1; }
constexpr size_t orbit_segff_offset(int n) { return orbit_seg_offset(n) + (size_t)(n - 1) * SEG_STRIDE; }
constexpr size_t orbit_table_doubles(int n) { return orbit_segff_offset(n) + (size_t)(n - 1) * SEGFF_STRIDE; }

GSLC_HD int orbit_piece(const Orbit& o, double t) {
    // core/Linspace.icc:77-89 search(t) - 2, clamped (InterpolateOrbit.icc:18-19)
    int idx = (int)((t - o.t0) * o.inv_spacing + 1) - 2;
    idx = idx < 0 ? 0 : idx;
    idx = idx > o.n - 4 ? o.n - 4 : idx;
    return idx;
}

// core/detail/InterpolateOrbit.icc:111-155 (interpolateOrbitLegendre): the
// 9-point Lagrange interpolant of the state vectors' positions and, apart,
// of their velocities, in the reference's operation order (no contraction);
// Linspace::search and operator[] (core/Linspace.icc:77-89) for the window.
// o.coef: positions (3n doubles), then velocities (3n).  t in the orbit span.
GSLC_HD void orbit_eval_legendre(const Orbit& o, double t, V3& pos, V3& vel) {
    const double last = dadd(o.t0, dmul((double)(o.n - 1), o.spacing));
    int search = o.n;
    if (t < o.t0) search = 0;
    else if (!(t > last)) search = (int)dadd(ddiv(dsub(t, o.t0), o.spacing), 1.0);
    int idx = search - 5;
    idx = idx < 0 ? 0 : idx;
    idx = idx > o.n - 9 ? o.n - 9 : idx;
    const double t_lo = dadd(o.t0, dmul((double)idx, o.spacing));
    const double t_hi = dadd(o.t0, dmul((double)(idx + 8), o.spacing));
    const double trel = ddiv(dmul(8.0, dsub(t, t_lo)), dsub(t_hi, t_lo));
    double teller = 1.0;
#pragma unroll
    for (int i = 0; i < 9; ++i) teller = dmul(teller, dsub(trel, (double)i));
    const double* P = o.coef;
    const double* V = o.coef + 3 * (size_t)o.n;
    if (teller == 0.0) {
        const int i = idx + (int)trel;
        pos = {ld_ro(P + 3 * i), ld_ro(P + 3 * i + 1), ld_ro(P + 3 * i + 2)};
        vel = {ld_ro(V + 3 * i), ld_ro(V + 3 * i + 1), ld_ro(V + 3 * i + 2)};
        return;
    }
    constexpr double noemer[9] = {40320.0, -5040.0, 1440.0, -720.0, 576.0, -720.0, 1440.0, -5040.0, 40320.0};
    double px = 0.0, py = 0.0, pz = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double coeff = ddiv(ddiv(teller, noemer[i]), dsub(trel, (double)i));
        const double* pi = P + 3 * (size_t)(idx + i);
        const double* vi = V + 3 * (size_t)(idx + i);
        px = dadd(px, dmul(coeff, ld_ro(pi)));
        py = dadd(py, dmul(coeff, ld_ro(pi + 1)));
        pz = dadd(pz, dmul(coeff, ld_ro(pi + 2)));
        vx = dadd(vx, dmul(coeff, ld_ro(vi)));
        vy = dadd(vy, dmul(coeff, ld_ro(vi + 1)));
        vz = dadd(vz, dmul(coeff, ld_ro(vi + 2)));
    }
    pos = {px, py, pz};
    vel = {vx, vy, vz};
}

GSLC_HD void orbit_eval(const Orbit& o, double t, V3& pos, V3& vel) {
    if (o.legendre) {
        orbit_eval_legendre(o, t, pos, vel);
        return;
    }
    const int idx = orbit_piece(o, t);
    const double* c = o.coef + (long)idx * ORB_STRIDE;
    const double tidx = o.t0 + idx * o.spacing;
    const double u = (t - tidx) * o.inv_spacing - 1.5;
    double p[3], v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const double* a = c + 3 + d * 8;
        double acc = ld_ro(a + 7);
#pragma unroll
        for (int k = 6; k >= 0; --k) acc = acc * u + ld_ro(a + k);
        p[d] = ld_ro(c + d) + acc;
        const double* b = c + 27 + d * 7;
        double vacc = ld_ro(b + 6);
#pragma unroll
        for (int k = 5; k >= 0; --k) vacc = vacc * u + ld_ro(b + k);
        v[d] = vacc;
    }
    pos = {p[0], p[1], p[2]};
    vel = {v[0], v[1], v[2]};
}

// Segment of orbit_piece(t) = pc at piece coordinate u; u becomes the
// segment coordinate w (exact: u + 1 and u - 1 on these ranges).
GSLC_HD int orbit_segment(const Orbit& o, int pc, double& u) {
    if (pc == 0 && u < -0.5) { u += 1.0; return 0; }
    if (pc == o.n - 4 && u >= 0.5) { u -= 1.0; return o.n - 2; }
    return pc + 1;
}


GSLC_HD double seg_poly(const double* c, int deg, double w) {
    double acc = ld_gen(c + deg);
    for (int k = deg - 1; k >= 0; --k) acc = fma(acc, w, ld_gen(c + k));
    return acc;
}

// Iterations 1.. of geo2rdr's zero-Doppler Newton solve
// (geometry/detail/Geo2Rdr.icc:114-179 with fdop = fdopder = 0): the same
// iterates t <- t - fn/fn', fn = (xyz - pos).vel, fn' = -|vel|^2, with fn
// formed on the segment tables (Orbit::seg) instead of subtracting the
// interpolated position: fn(w) = D.v(w) - H(w) with D = xyz - P_ref is one
// polynomial whose coefficients k <= 6 are D.b_k - h_k (formed when the
// iterate enters a segment) and whose others are -h_k (H truncated where its
// tail stops mattering; the degree-6 term too where it does not matter,
// Orbit::seg_r6); 1/|vel|^2 is G(w).  Inside a segment the iterate is
// carried by its coordinate w alone, t = t_j + (w + 1/2) spacing being
// formed where it is needed (segment changes and the returned iterate).
// Rounding differs from the direct form by ~1e-13 s in azimuth time, below
// the reference's own orbit interpolation noise (~1e-11 s).
// seg: the segment tables (Orbit::seg, or a copy of them in shared memory).
GSLC_HD bool geo2rdr_zero_doppler_seg(const Orbit& o, const double* seg, V3 xyz, double thr, int maxiter, double& t,
                                       double dt, double& R) {
    int cur = -1;
    double D[3] = {0.0, 0.0, 0.0};
    double cf[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // fn(w) coefficients 0..6
    double w = 0.0;
    const double* c = seg;
    const int nh = o.seg_nh;
    // |dt| < thr as a bit compare (thr <= 0 or NaN: never, as the FP64
    // test); thr > 0.0 from its bits as well
    const uint64_t tb = dbits(thr);
    const uint64_t thr_bits = ((int64_t)tb > 0 && tb <= (uint64_t)DKEY_INF) ? tb : 0ull;
    // the orbit's time span as order keys (the range test below)
    const int64_t k_t0 = dkey(o.t0), k_tend = dkey(o.t_end);
    // G(w) = 1/|vel|^2 changes by ~5e-6 of itself per second of the
    // iterate's travel.  Once a step falls below 0.1 s the iterate travels
    // at most ~0.014 s more (the steps shrink by ~0.12 each), so the last G
    // stays within ~7e-8 of the current one and is reused: each later step
    // changes by at most that fraction of itself, a change the contraction
    // shrinks to ~1e-14 s in the returned iterate, well below the ~1e-13 s
    // the segment form already differs by; the fixed point fn = 0 does not
    // depend on G at all.
    double g = 0.0;
    bool g_fresh = false;
    double tj = 0.0;                     // start time of segment cur
    for (int i = 1; i < maxiter; ++i) {
        // Inside an interior segment the iterate moves as w -= dt / spacing
        // (~1e-15 s from the exact coordinate); entering a segment, leaving
        // it, and on the first and last segment (the orbit's time span) the
        // time, the span check, the piece and w come from it as orbit
        // interpolation forms them.
        w -= dt * o.inv_spacing;
        // w in [-0.5, 0.5): |w| < 0.5 or w == -0.5
        const uint64_t wb = dbits(w);
        const bool in_seg = (wb & DMAG) < DBITS_HALF || wb == DBITS_MINUS_HALF;
        if (cur <= 0 || cur >= o.n - 2 || !in_seg) {
            if (cur < 0) t -= dt;        // the first step, from the caller's iterate
            else t = tj + (w + 0.5) * o.spacing;
            const int64_t kt = dkey(t);
            if (!(kt >= k_t0 && kt <= k_tend)) return false;  // FillNaN -> no convergence
            // orbit_piece(o, t) with the truncation from the bits (the
            // argument is at least 1 here, t >= t0), then t_idx, the start
            // of segment pc, from the tables
            uint64_t fb;
            const int32_t tr = split_bits((t - o.t0) * o.inv_spacing + 1, fb);
            int pc = tr - 2;
            pc = pc < 0 ? 0 : pc;
            pc = pc > o.n - 4 ? o.n - 4 : pc;
            const double tidx = ld_gen(seg + (int64_t)pc * SEG_STRIDE + SEG_T);
            w = (t - tidx) * o.inv_spacing - 1.5;
            const int j = orbit_segment(o, pc, w);
            c = seg + (int64_t)j * SEG_STRIDE;
            if (j != cur) {
                cur = j;
                tj = ld_gen(c + SEG_T);
                D[0] = xyz.x - ld_gen(c + 0);
                D[1] = xyz.y - ld_gen(c + 1);
                D[2] = xyz.z - ld_gen(c + 2);
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    if (k == 6 && !o.seg_r6) break;
                    const double dv = fma(D[0], ld_gen(c + SEG_B + k), fma(D[1], ld_gen(c + SEG_B + 7 + k),
                                                                         D[2] * ld_gen(c + SEG_B + 14 + k)));
                    cf[k] = k <= nh ? dv - ld_gen(c + SEG_H + k) : dv;
                }
            }
        }
        double fn;
        if (o.seg_div) {
            // G did not converge on some segment: the direct form, dividing by -|vel|^2
            double v[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double* b = c + SEG_B + d * 7;
                double acc = ld_gen(b + 6);
#pragma unroll
                for (int k = 5; k >= 0; --k) acc = fma(acc, w, ld_gen(b + k));
                v[d] = acc;
            }
            fn = fma(D[0], v[0], fma(D[1], v[1], D[2] * v[2])) - seg_poly(c + SEG_H, nh, w);
            dt = fn / (-(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
        } else {
            double acc;
            if (o.seg_r6) {
                acc = cf[6];
                if (nh > 6) {
                    acc = -ld_gen(c + SEG_H + nh);
                    for (int k = nh - 1; k >= 7; --k) acc = fma(acc, w, -ld_gen(c + SEG_H + k));
                    acc = fma(acc, w, cf[6]);
                }
                acc = fma(acc, w, cf[5]);
            } else {
                acc = cf[5];
            }
#pragma unroll
            for (int k = 4; k >= 0; --k) acc = fma(acc, w, cf[k]);
            fn = acc;
            if (!g_fresh) g = seg_poly(c + SEG_G, o.seg_ng, w);
            dt = -fn * g;
            g_fresh = (dbits(dt) & DMAG) < DBITS_0P1;
        }
        if ((dbits(dt) & DMAG) < thr_bits) {
            t = tj + (w + 0.5) * o.spacing;
            double r[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const double* a = c + SEG_A + d * 8;
                double acc = o.seg_a7 ? fma(ld_gen(a + 7), w, ld_gen(a + 6)) : ld_gen(a + 6);
#pragma unroll
                for (int k = 5; k >= 0; --k) acc = fma(acc, w, ld_gen(a + k));
                r[d] = D[d] - acc;
            }
            R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            return true;
        }
    }
    return false;
}

// Iterations 1.. of the zero-Doppler Newton solve with the orbit
// interpolated at every iterate (geometry/detail/Geo2Rdr.icc:114-179 with
// fdop = fdopder = 0, where fn = rvec.vel and fn' = -vel.vel exactly): the
// form for orbits the segment tables do not hold (Legendre).  Same
// arguments as geo2rdr_zero_doppler_seg without the tables.
GSLC_HD bool geo2rdr_zero_doppler_orbit(const Orbit& o, V3 xyz, double thr, int maxiter, double& t, double dt,
                                        double& R) {
    for (int i = 1; i < maxiter; ++i) {
        t -= dt;
        if (!(t >= o.t0 && t <= o.t_end)) return false;   // FillNaN -> no convergence
        V3 pos, vel;
        orbit_eval(o, t, pos, vel);
        const V3 rvec = vsub(xyz, pos);
        R = vnorm(rvec);
        dt = vdot(rvec, vel) / (-vdot(vel, vel));
        if (fabs(dt) < thr) return true;
    }
    return false;
}

// ---- float-float (double-word FP32) arithmetic ------------------------------
// Dekker (1971) products and Knuth's TwoSum, in the double-word forms of
// Joldes, Muller & Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic" (ACM TOMS 44(2), 2017):
// relative error of add/mul about 2^-44.  Only plain IEEE add/mul and fmaf
// are used, so nvcc cannot reassociate them.
struct ff { float hi, lo; };

#if defined(__CUDACC__)
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_from_double(double d) {
    const float hi = __double2float_rn(d);
    return {hi, __double2float_rn(d - (double)hi)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ ff ff_add(ff x, ff y) {                   // AccurateDWPlusDW
    ff s = ff_two_sum(x.hi, y.hi);
    const ff t = ff_two_sum(x.lo, y.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = ff_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_mul(ff x, ff y) {                   // DWTimesDW
    const float p = __fmul_rn(x.hi, y.hi);
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, e);
    e = fmaf(x.lo, y.hi, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_mul_f(ff x, float y) {              // DWTimesFP1
    const float p = __fmul_rn(x.hi, y);
    float e = fmaf(x.hi, y, -p);
    e = fmaf(x.lo, y, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_fma(ff x, ff y, ff z) { return ff_add(ff_mul(x, y), z); }
__device__ __forceinline__ ff ff_div(ff a, ff b) {                   // DWDivDW (long division)
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const ff r = ff_add(a, ff_neg(ff_mul(b, {q1, 0.f})));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    return ff_fast_two_sum(q1, q2);
}
#endif

// ---- Biquintic spline, FP32, exact reference order -------------------------
// core/Spline2dInterpolator.cpp:89-108 (_initSpline) for n = 6.  p[i], q[i]
// depend on nothing but n; the host computes them with the same FP32 ops.
struct SplineConst {
    float p[5], q[5];       // FP32 recurrence (core/Spline2dInterpolator.cpp)
    double pd[5];           // FP64 p of the CUDA interpolator (cuda/core/gpuSpline2dInterpolator.cu)
    float qd[5];            // its Q, stored to FP32
};

GSLC_HD void init_spline6(const float Y[6], float R[6], const SplineConst& k) {
    R[0] = 0.0f;
#pragma unroll
    for (int i = 1; i < 5; ++i) {
        const float t = fadd(fsub(Y[i + 1], fmul(2.0f, Y[i])), Y[i - 1]);
        R[i] = fmul(fsub(fmul(3.0f, t), fmul(0.5f, R[i - 1])), k.p[i]);
    }
    R[5] = 0.0f;
#pragma unroll
    for (int i = 4; i > 0; --i) R[i] = fadd(fmul(k.q[i], R[i + 1]), R[i]);
}

// cuda/core/gpuSpline2dInterpolator.cu:85-101 (_initSpline) for T = float
// and n = 6: the double literals promote parts of each expression to FP64,
// and the results are stored back to FP32; every operation rounds once.
GSLC_HD void init_spline6_gpu(const float Y[6], float R[6], const SplineConst& k) {
    R[0] = 0.0f;
#pragma unroll
    for (int i = 1; i < 5; ++i) {
        const float s = fmul(3.0f, fadd(fsub(Y[i + 1], fmul(2.0f, Y[i])), Y[i - 1]));
        R[i] = (float)dmul(dsub((double)s, dmul(0.5, (double)R[i - 1])), k.pd[i]);
    }
    R[5] = 0.0f;
#pragma unroll
    for (int i = 4; i > 0; --i) R[i] = fadd(fmul(k.qd[i], R[i + 1]), R[i]);
}

// cuda/core/gpuSpline2dInterpolator.cu:103-117 (_spline) on its in-range
// branch (x in [2, 3), j = 2), mixed precision as written there.
GSLC_HD float spline6_at_gpu(double x, const float Y[6], const float R[6]) {
    const double xx = dsub(x, 2.0);
    const double t0 = dsub(dsub((double)fsub(Y[2], Y[1]), ddiv((double)R[1], 3.0)), ddiv((double)R[2], 6.0));
    const float d6 = fdiv(fsub(R[2], R[1]), 6.0f);
    const double t1 = dmul(xx, dadd(ddiv((double)R[1], 2.0), dmul(xx, (double)d6)));
    return (float)dadd((double)Y[1], dmul(xx, dadd(t0, t1)));
}

// core/Spline2dInterpolator.cpp:69-87 (_spline) on the branch every in-range
// DEM point takes: x - j0 lies in [2, 3), so j = 2.
GSLC_HD float spline6_at(float xx, const float Y[6], const float R[6]) {
    const float t0 = fsub(fsub(fsub(Y[2], Y[1]), fdiv(R[1], 3.0f)), fdiv(R[2], 6.0f));
    const float t1 = fmul(xx, fadd(fmul(R[1], 0.5f), fmul(xx, fdiv(fsub(R[2], R[1]), 6.0f))));
    return fadd(Y[1], fmul(xx, fadd(t0, t1)));
}

}  // namespace gslc
