// CPU oracle for SLC geocoding — TEST INFRASTRUCTURE ONLY (see gslc_oracle.h).
//
// Every function cites the reference file:line it restates.  Operation order
// is kept where the reference computes in FP32 (DEM spline, deramp phase,
// sinc accumulation, complex products), because FP32 rounding there moves the
// flattening phase by more than the parity tolerance.  Compile with
// -ffp-contract=off.
#include "gslc_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;
int fail(const std::string& m) { g_err = m; return 1; }

constexpr int SINC_HALF = 4;    // core/Constants.h:32
constexpr int SINC_LEN = 8;     // core/Constants.h:33
constexpr int SINC_ONE = 9;     // core/Constants.h:34
constexpr int SINC_SUB = 8192;  // core/Constants.h:35
const double NaN = std::numeric_limits<double>::quiet_NaN();

struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// complex<float> product the way GCC lowers it for finite operands:
// (ac - bd) + (ad + bc)i, each product rounded (no FMA).
struct cf { float re, im; };
inline cf cmul(cf a, cf b) {
    float ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    return {ac - bd, ad + bc};
}

// ---------------------------------------------------------------- Orbit
// core/Linspace.h:56 operator[], core/Linspace.icc:77-89 search
inline double orb_time(const orc_orbit* o, int i) { return o->t0 + i * o->spacing; }
inline int orb_search(const orc_orbit* o, double t) {
    double first = o->t0, last = orb_time(o, o->n - 1);
    if (o->spacing >= 0) {
        if (t < first) return 0;
        if (t > last) return o->n;
    } else {
        if (t > first) return 0;
        if (t < last) return o->n;
    }
    return (int)((t - first) / o->spacing + 1);
}
inline V3 orb_pos(const orc_orbit* o, int i) { return {o->pos[3*i], o->pos[3*i+1], o->pos[3*i+2]}; }
inline V3 orb_vel(const orc_orbit* o, int i) { return {o->vel[3*i], o->vel[3*i+1], o->vel[3*i+2]}; }

// core/detail/InterpolateOrbit.icc:10-109
void hermite(const orc_orbit* o, double t, V3* position, V3* velocity) {
    int idx = orb_search(o, t) - 2;
    idx = std::min(std::max(idx, 0), o->n - 4);
    double f1[4], f0[4], h[4], hdot[4], g1[4], g0[4];
    for (int i = 0; i < 4; ++i) f1[i] = t - orb_time(o, idx + i);
    for (int i = 0; i < 4; ++i) {
        double sum = 0.;
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            sum += 1. / (orb_time(o, idx + i) - orb_time(o, idx + j));
        }
        f0[i] = 1. - 2. * sum * (t - orb_time(o, idx + i));
    }
    for (int i = 0; i < 4; ++i) {
        h[i] = 1.;
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            h[i] *= (t - orb_time(o, idx + j)) / (orb_time(o, idx + i) - orb_time(o, idx + j));
        }
    }
    if (position) {
        V3 p{0., 0., 0.};
        for (int i = 0; i < 4; ++i) {
            V3 P = orb_pos(o, idx + i), Vv = orb_vel(o, idx + i);
            // h*h*(P*f0 + V*f1), Vec3 ops are component-wise
            double hh = h[i] * h[i];
            p.x += hh * (P.x * f0[i] + Vv.x * f1[i]);
            p.y += hh * (P.y * f0[i] + Vv.y * f1[i]);
            p.z += hh * (P.z * f0[i] + Vv.z * f1[i]);
        }
        *position = p;
    }
    if (!velocity) return;
    for (int i = 0; i < 4; ++i) {
        hdot[i] = 0.;
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            double prod = 1. / (orb_time(o, idx + i) - orb_time(o, idx + j));
            for (int k = 0; k < 4; ++k) {
                if (k == i || k == j) continue;
                prod *= (t - orb_time(o, idx + k)) / (orb_time(o, idx + i) - orb_time(o, idx + k));
            }
            hdot[i] += prod;
        }
    }
    for (int i = 0; i < 4; ++i) g1[i] = h[i] + 2. * hdot[i] * (t - orb_time(o, idx + i));
    for (int i = 0; i < 4; ++i) {
        double sum = 0.;
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            sum += 1. / (orb_time(o, idx + i) - orb_time(o, idx + j));
        }
        g0[i] = 2. * (f0[i] * hdot[i] - sum * h[i]);
    }
    V3 v{0., 0., 0.};
    for (int i = 0; i < 4; ++i) {
        V3 P = orb_pos(o, idx + i), Vv = orb_vel(o, idx + i);
        v.x += h[i] * (P.x * g0[i] + Vv.x * g1[i]);
        v.y += h[i] * (P.y * g0[i] + Vv.y * g1[i]);
        v.z += h[i] * (P.z * g0[i] + Vv.z * g1[i]);
    }
    *velocity = v;
}

// core/detail/InterpolateOrbit.icc:111-155
void legendre(const orc_orbit* o, double t, V3* position, V3* velocity) {
    int idx = orb_search(o, t) - 5;
    idx = std::min(std::max(idx, 0), o->n - 9);
    double trel = 8. * (t - orb_time(o, idx)) / (orb_time(o, idx + 8) - orb_time(o, idx));
    double teller = 1.;
    for (int i = 0; i < 9; ++i) teller *= trel - i;
    if (teller == 0.) {
        int i = (int)trel;
        if (position) *position = orb_pos(o, idx + i);
        if (velocity) *velocity = orb_vel(o, idx + i);
        return;
    }
    static const double noemer[9] = {40320.0, -5040.0, 1440.0, -720.0, 576.0,
                                      -720.0, 1440.0, -5040.0, 40320.0};
    V3 p{0., 0., 0.}, v{0., 0., 0.};
    for (int i = 0; i < 9; ++i) {
        double coeff = (teller / noemer[i]) / (trel - i);
        V3 P = orb_pos(o, idx + i), Vv = orb_vel(o, idx + i);
        p.x += coeff * P.x; p.y += coeff * P.y; p.z += coeff * P.z;
        v.x += coeff * Vv.x; v.y += coeff * Vv.y; v.z += coeff * Vv.z;
    }
    if (position) *position = p;
    if (velocity) *velocity = v;
}

// core/detail/InterpolateOrbit.icc:157-193 (border mode FillNaN);
// returns 0 on success.
int orbit_interp(const orc_orbit* o, double t, V3* pos, V3* vel) {
    int minsv = o->method == 1 ? 9 : 4;
    if (o->n < minsv) return 2;
    if (t < o->t0 || t > orb_time(o, o->n - 1)) {
        if (pos) *pos = {NaN, NaN, NaN};
        if (vel) *vel = {NaN, NaN, NaN};
        return 1;
    }
    if (o->method == 1) legendre(o, t, pos, vel); else hermite(o, t, pos, vel);
    return 0;
}

// ---------------------------------------------------------------- LUT2d
// core/LUT2d.h:84-95
bool lut_contains(const orc_lut2d* l, double y, double x) {
    if (!l->have_data) return true;
    const double i = (x - l->x0) / l->dx;
    const double j = (y - l->y0) / l->dy;
    return (i >= 0.0 && i <= l->nx - 1.0) && (j >= 0.0 && j <= l->ny - 1.0);
}

// core/BilinearInterpolator.cpp:12-49 (U = double)
double bilinear(const double* z, int nx, double x, double y) {
    int x1 = (int)std::floor(x), x2 = (int)std::ceil(x);
    int y1 = (int)std::floor(y), y2 = (int)std::ceil(y);
    double q11 = z[(size_t)y1 * nx + x1], q12 = z[(size_t)y2 * nx + x1];
    double q21 = z[(size_t)y1 * nx + x2], q22 = z[(size_t)y2 * nx + x2];
    if ((y1 == y2) && (x1 == x2)) return q11;
    if (y1 == y2)
        return ((double)((x2 - x) / (x2 - x1)) * q11) + ((double)((x - x1) / (x2 - x1)) * q21);
    if (x1 == x2)
        return ((double)((y2 - y) / (y2 - y1)) * q11) + ((double)((y - y1) / (y2 - y1)) * q12);
    const double den = (double)((x2 - x1) * (y2 - y1));
    return ((q11 * (double)((x2 - x) * (y2 - y))) / den) +
           ((q21 * (double)((x - x1) * (y2 - y))) / den) +
           ((q12 * (double)((x2 - x) * (y - y1))) / den) +
           ((q22 * (double)((x - x1) * (y - y1))) / den);
}

// core/NearestNeighborInterpolator.cpp:12-22
double nearest(const double* z, int nx, double x, double y) {
    long row = (long)std::round(y), col = (long)std::round(x);
    return z[(size_t)row * nx + col];
}

// core/BicubicInterpolator.cpp:37-42 (cubicInterpolate, T = double)
double cubic_interpolate(double p0, double p1, double p2, double p3, double tfrac) {
    const double tconj = 1. - tfrac;
    return (tfrac * (p2 - p0 * (tconj * tconj) + (p2 * (tconj * 3. + 1.) - p3 * tconj) * tfrac) +
            p1 * (tfrac * tfrac * (tfrac * 3. - 5.) + 2.)) / 2.;
}

// core/BicubicInterpolator.cpp:47-64 (U = double).  The reference reads the
// 4 x 4 neighbourhood unchecked, outside its matrix at the edge rows and
// columns (undefined there); here those reads are clamped to the matrix.
double bicubic(const double* z, int ny, int nx, double x, double y) {
    const int x0 = (int)std::floor(x), y0 = (int)std::floor(y);
    auto at = [&](int r, int c) {
        r = std::min(std::max(r, 0), ny - 1);
        c = std::min(std::max(c, 0), nx - 1);
        return z[(size_t)r * nx + c];
    };
    double intp[4];
    for (int i = -1; i < 3; i++)
        intp[i + 1] = cubic_interpolate(at(y0 + i, x0 - 1), at(y0 + i, x0), at(y0 + i, x0 + 1), at(y0 + i, x0 + 2),
                                        x - x0);
    return cubic_interpolate(intp[0], intp[1], intp[2], intp[3], y - y0);
}

template <typename U>
U spline2d(const U* z, int ny, int nx, double x, double y);
double sinc2d_double(const double* z, int rows, int cols, double x, double y);

// core/LUT2d.cpp:124-158 (out-of-bounds only logs; index is clamped), with
// the interpolator of the table's method (core/LUT2d.cpp _setInterpolator):
// 0 sinc, 1 bilinear, 2 bicubic, 3 nearest, 4 biquintic
double lut_eval(const orc_lut2d* l, double y, double x) {
    double value = l->ref_value;
    if (!l->have_data) return value;
    double x_idx = (x - l->x0) / l->dx;
    double y_idx = (y - l->y0) / l->dy;
    x_idx = std::min(std::max(x_idx, 0.0), l->nx - 1.0);
    y_idx = std::min(std::max(y_idx, 0.0), l->ny - 1.0);
    switch (l->method) {
        case 0: return sinc2d_double(l->data, l->ny, l->nx, x_idx, y_idx);
        case 2: return bicubic(l->data, l->ny, l->nx, x_idx, y_idx);
        case 3: return nearest(l->data, l->nx, x_idx, y_idx);
        case 4: return spline2d<double>(l->data, l->ny, l->nx, x_idx, y_idx);
        default: return bilinear(l->data, l->nx, x_idx, y_idx);
    }
}

// ---------------------------------------------------------------- Poly2d
// core/Poly2d.cpp:8-24
double poly_eval(const orc_poly2d* p, double y, double x) {
    double xval = (x - p->x_mean) / p->x_norm;
    double yval = (y - p->y_mean) / p->y_norm;
    double scalex, scaley = 1., val = 0.;
    for (int i = 0; i <= p->y_order; i++, scaley *= yval) {
        scalex = 1.;
        for (int j = 0; j <= p->x_order; j++, scalex *= xval)
            val += scalex * scaley * p->coeffs[i * (p->x_order + 1) + j];
    }
    return val;
}

double azrg_eval(const orc_azrg* f, double y, double x) {
    return f->kind == 1 ? poly_eval(&f->poly, y, x) : lut_eval(&f->lut, y, x);
}

// ---------------------------------------------------------------- Ellipsoid
// core/Ellipsoid.h:117-120 (rEast) and :177-190 (lonLatToXyz)
V3 lonlat_to_xyz(double a, double e2, V3 llh) {
    double re = a / std::sqrt(1.0 - (e2 * std::pow(std::sin(llh.y), 2)));
    V3 xyz;
    xyz.x = (re + llh.z) * std::cos(llh.y) * std::cos(llh.x);
    xyz.y = (re + llh.z) * std::cos(llh.y) * std::sin(llh.x);
    xyz.z = ((re * (1.0 - e2)) + llh.z) * std::sin(llh.y);
    return xyz;
}

// ---------------------------------------------------------------- Projections
constexpr double WGS84_A = 6378137.0;                  // core/Constants.h:41
constexpr double WGS84_E2 = 0.006694379990141317;      // core/Constants.h:44

// core/Projections.cpp:33-42
double clens(const double* a, int size, double real) {
    const double* p;
    double hr, hr1, hr2;
    for (p = a + size, hr2 = 0., hr1 = *(--p), hr = 0.; a - p; hr2 = hr1, hr1 = hr)
        hr = -hr2 + (2. * hr1 * std::cos(real)) + *(--p);
    return std::sin(real) * hr;
}

// core/Projections.cpp:54-74
double clenS(const double* a, int size, double real, double imag, double& R, double& I) {
    const double* p;
    double hr, hr1, hr2, hi, hi1, hi2;
    for (p = a + size, hr2 = 0., hi2 = 0., hi1 = 0., hr1 = *(--p), hi1 = 0., hr = 0., hi = 0.;
         a - p; hr2 = hr1, hi2 = hi1, hr1 = hr, hi1 = hi) {
        hr = -hr2 + (2. * hr1 * std::cos(real) * std::cosh(imag)) -
             (-2. * hi1 * std::sin(real) * std::sinh(imag)) + *(--p);
        hi = -hi2 + (-2. * hr1 * std::sin(real) * std::sinh(imag)) +
             (2. * hi1 * std::cos(real) * std::cosh(imag));
    }
    R = (std::sin(real) * std::cosh(imag) * hr) - (std::cos(real) * std::sinh(imag) * hi);
    I = (std::sin(real) * std::cosh(imag) * hi) + (std::cos(real) * std::sinh(imag) * hr);
    return R;
}

struct UTM {
    int zone; bool isnorth;
    double lon0, Qn, Zb, cgb[6], cbg[6], utg[6], gtu[6];
};

// core/Projections.cpp:80-170
bool utm_setup(int code, UTM& u) {
    if (code > 32600 && code <= 32660) { u.zone = code - 32600; u.isnorth = true; }
    else if (code > 32700 && code <= 32760) { u.zone = code - 32700; u.isnorth = false; }
    else return false;
    u.lon0 = ((u.zone - 0.5) * (M_PI / 30.)) - M_PI;
    double f = WGS84_E2 / (1. + std::sqrt(1 - WGS84_E2));
    double n = f / (2. - f);
    u.cgb[0] = n * (2 + n * ((-2. / 3.) + n * (-2 + n * ((116. / 45.) + n * ((26. / 45.) + n * (-2854. / 675.))))));
    u.cbg[0] = n * (-2 + n * ((2. / 3.) + n * ((4. / 3.) + n * ((-82. / 45.) + n * ((32. / 45.) + n * (4642. / 4725.))))));
    u.cgb[1] = std::pow(n, 2) * ((7. / 3.) + n * ((-8. / 5.) + n * ((-227. / 45.) + n * ((2704. / 315.) + n * (2323. / 945.)))));
    u.cbg[1] = std::pow(n, 2) * ((5. / 3.) + n * ((-16. / 15.) + n * ((-13. / 9.) + n * ((904. / 315.) + n * (-1522. / 945.)))));
    u.cgb[2] = std::pow(n, 3) * ((56. / 15.) + n * ((-136. / 35.) + n * ((-1262. / 105.) + n * (73814. / 2835.))));
    u.cbg[2] = std::pow(n, 3) * ((-26. / 15.) + n * ((34. / 21.) + n * ((8. / 5.) + n * (-12686. / 2835.))));
    u.cgb[3] = std::pow(n, 4) * ((4279. / 630.) + n * ((-332. / 35.) + n * (-399572 / 14175.)));
    u.cbg[3] = std::pow(n, 4) * ((1237. / 630.) + n * ((-12. / 5.) + n * (-24832. / 14175.)));
    u.cgb[4] = std::pow(n, 5) * ((4174. / 315.) + n * (-144838. / 6237.));
    u.cbg[4] = std::pow(n, 5) * ((-734. / 315.) + n * (109598. / 31185.));
    u.cgb[5] = std::pow(n, 6) * (601676. / 22275.);
    u.cbg[5] = std::pow(n, 6) * (444337. / 155925.);
    u.Qn = (0.9996 / (1. + n)) * (1. + n * n * ((1. / 4.) + n * n * ((1. / 64.) + ((n * n) / 256.))));
    u.utg[0] = n * (-.5 + n * ((2. / 3.) + n * ((-37. / 96.) + n * ((1. / 360.) + n * ((81. / 512.) + n * (-96199. / 604800.))))));
    u.gtu[0] = n * (.5 + n * ((-2. / 3.) + n * ((5. / 16.) + n * ((41. / 180.) + n * ((-127. / 288.) + n * (7891. / 37800.))))));
    u.utg[1] = std::pow(n, 2) * ((-1. / 48.) + n * ((-1. / 15.) + n * ((437. / 1440.) + n * ((-46. / 105.) + n * (1118711. / 3870720.)))));
    u.gtu[1] = std::pow(n, 2) * ((13. / 48.) + n * ((-3. / 5.) + n * ((557. / 1440.) + n * ((281. / 630.) + n * (-1983433. / 1935360.)))));
    u.utg[2] = std::pow(n, 3) * ((-17. / 480.) + n * ((37. / 840.) + n * ((209. / 4480.) + n * (-5569. / 90720.))));
    u.gtu[2] = std::pow(n, 3) * ((61. / 240.) + n * ((-103. / 140.) + n * ((15061. / 26880.) + n * (167603. / 181440.))));
    u.utg[3] = std::pow(n, 4) * ((-4397. / 161280.) + n * ((11. / 504.) + n * (830251. / 7257600.)));
    u.gtu[3] = std::pow(n, 4) * ((49561. / 161280.) + n * ((-179. / 168.) + n * (6601661. / 7257600.)));
    u.utg[4] = std::pow(n, 5) * ((-4583. / 161280.) + n * (108847. / 3991680.));
    u.gtu[4] = std::pow(n, 5) * ((34729. / 80640.) + n * (-3418889. / 1995840.));
    u.utg[5] = std::pow(n, 6) * (-20648693. / 638668800.);
    u.gtu[5] = std::pow(n, 6) * (212378941. / 319334400.);
    double Z = clens(u.cbg, 6, 0.);
    u.Zb = -u.Qn * (Z + clens(u.gtu, 6, 2 * Z));
    return true;
}

// core/Projections.cpp:172-198
int utm_forward(const UTM& u, V3 llh, V3& out) {
    double gauss = clens(u.cbg, 6, 2. * llh.y) + llh.y;
    double lam = llh.x - u.lon0;
    double Cn = std::atan2(std::sin(gauss), std::cos(lam) * std::cos(gauss));
    double Ce = std::atan2(std::sin(lam) * std::cos(gauss),
                           std::hypot(std::sin(gauss), std::cos(gauss) * std::cos(lam)));
    Ce = std::asinh(std::tan(Ce));
    double dCn, dCe;
    Cn += clenS(u.gtu, 6, 2 * Cn, 2 * Ce, dCn, dCe);
    Ce += dCe;
    if (std::fabs(Ce) <= 2.623395162778) {
        out.x = (u.Qn * Ce * WGS84_A) + 500000.;
        out.y = (((u.Qn * Cn) + u.Zb) * WGS84_A) + (u.isnorth ? 0. : 10000000.);
        out.z = llh.z;
        return 0;
    }
    return 1;
}

// core/Projections.cpp:200-232
int utm_inverse(const UTM& u, V3 in, V3& llh) {
    double Cn = (in.y - (u.isnorth ? 0. : 10000000.)) / WGS84_A;
    double Ce = (in.x - 500000.) / WGS84_A;
    Cn = (Cn - u.Zb) / u.Qn;
    Ce /= u.Qn;
    if (std::fabs(Ce) <= 2.623395162778) {
        double dCn, dCe;
        Cn += clenS(u.utg, 6, 2 * Cn, 2 * Ce, dCn, dCe);
        Ce = std::atan(std::sinh(Ce + dCe));
        double sinCe = std::sin(Ce);
        double cosCe = std::cos(Ce);
        Ce = std::atan2(sinCe, cosCe * std::cos(Cn));
        Cn = std::atan2(std::sin(Cn) * cosCe, std::hypot(sinCe, cosCe * std::cos(Cn)));
        llh.x = Ce + u.lon0;
        llh.y = clens(u.cgb, 6, 2 * Cn) + Cn;
        llh.z = in.z;
        return 0;
    }
    return 1;
}

// Projection object: LonLat (core/Projections.h:127-140) or UTM.
struct Proj {
    int epsg = 0; UTM utm{};
    bool init(int code) {
        epsg = code;
        if (code == 4326) return true;
        if (code > 32600 && code < 32800) return utm_setup(code, utm);
        return false;
    }
    int forward(V3 llh, V3& out) const {
        if (epsg == 4326) {
            out.x = llh.x * 180.0 / M_PI; out.y = llh.y * 180.0 / M_PI; out.z = llh.z;
            return 0;
        }
        return utm_forward(utm, llh, out);
    }
    int inverse(V3 in, V3& llh) const {
        if (epsg == 4326) {
            llh.x = in.x * M_PI / 180.0; llh.y = in.y * M_PI / 180.0; llh.z = in.z;
            return 0;
        }
        return utm_inverse(utm, in, llh);
    }
};

// ---------------------------------------------------------------- Spline2d
// core/Spline2dInterpolator.cpp:89-108 (_initSpline)
template <typename U>
void init_spline(const U* Y, int n, U* R, U* Q) {
    Q[0] = U(0.0);
    R[0] = U(0.0);
    for (int i = 1; i < n - 1; ++i) {
        const U p = static_cast<U>(1.0) / (static_cast<U>(0.5) * Q[i - 1] + static_cast<U>(2.0));
        Q[i] = static_cast<U>(-0.5) * p;
        R[i] = (static_cast<U>(3.0) * (Y[i + 1] - static_cast<U>(2.0) * Y[i] + Y[i - 1]) -
                static_cast<U>(0.5) * R[i - 1]) * p;
    }
    R[n - 1] = U(0.0);
    for (int i = (n - 2); i > 0; --i) R[i] = Q[i] * R[i + 1] + R[i];
}

// core/Spline2dInterpolator.cpp:69-87 (_spline)
template <typename U>
U spline(double x, const U* Y, int n, const U* R) {
    const U denom = static_cast<U>(6.0);
    if (x < 1.0) {
        return Y[0] + static_cast<U>(x - 1.0) * (Y[1] - Y[0] - (R[1] / denom));
    } else if (x > n) {
        return Y[n - 1] + (static_cast<U>(x - n) * (Y[n - 1] - Y[n - 2] + (R[n - 2] / denom)));
    } else {
        int j = int(std::floor(x));
        U xx = static_cast<U>(x - j);
        U t0 = Y[j] - Y[j - 1] - (R[j - 1] / static_cast<U>(3.0)) - (R[j] / denom);
        U t1 = xx * ((R[j - 1] / static_cast<U>(2.0)) + (xx * ((R[j] - R[j - 1]) / denom)));
        return Y[j - 1] + (xx * (t0 + t1));
    }
}

// core/Spline2dInterpolator.cpp:32-67 (interp_impl, order 6)
template <typename U>
U spline2d(const U* z, int ny, int nx, double x, double y) {
    const int order = 6;
    int i0 = (int)y, j0 = (int)x;      // order even: truncation
    i0 = i0 - (order / 2) + 1;
    j0 = j0 - (order / 2) + 1;
    U A[order], R[order], Q[order], HC[order];
    for (int i = 0; i < order; ++i) {
        const int indi = std::min(std::max(i0 + i, 0), ny - 2);
        for (int j = 0; j < order; ++j) {
            const int indj = std::min(std::max(j0 + j, 0), nx - 2);
            A[j] = z[(size_t)(indi + 1) * nx + (indj + 1)];
        }
        init_spline(A, order, R, Q);
        HC[i] = spline(x - j0, A, order, R);
    }
    init_spline(HC, order, R, Q);
    return static_cast<U>(spline(y - i0, HC, order, R));
}

// ---------------------------------------------------------------- Sinc2d
// core/Sinc2dInterpolator.cpp:98-115 (_sinc_coef) and :12-40 (ctor)
struct SincTable {
    std::vector<double> k;   // [SINC_SUB][SINC_LEN]
    SincTable() : k((size_t)SINC_SUB * SINC_LEN) {
        const int filtercoef = SINC_SUB * SINC_LEN;
        std::vector<double> filter(filtercoef, 0.0);
        const double beta = 1.0, pedestal = 0.0;
        const double wgthgt = (1.0 - pedestal) / 2.0;
        const double soff = (filtercoef - 1.) / 2.;
        for (int i = 0; i < filtercoef; i++) {
            double wgt = (1. - wgthgt) + (wgthgt * std::cos((M_PI * (i - soff)) / soff));
            double s = (std::floor(i - soff) * beta) / (1. * SINC_SUB);
            double fct = ((s != 0.) ? (std::sin(M_PI * s) / (M_PI * s)) : 1.);
            filter[i] = fct * wgt;
        }
        for (size_t i = 0; i < (size_t)SINC_SUB; ++i) {
            double ssum = 0.0;
            for (size_t j = 0; j < (size_t)SINC_LEN; ++j) ssum += filter[i + SINC_SUB * j];
            for (size_t j = 0; j < (size_t)SINC_LEN; ++j) {
                filter[i + SINC_SUB * j] /= ssum;
                k[i * SINC_LEN + j] = filter[i + SINC_SUB * j];
            }
        }
    }
};
const SincTable& sinc_table() { static SincTable t; return t; }

// core/Sinc2dInterpolator.cpp:45-96 for U = complex<float>; the chip is the
// 9x9 Matrix built in geocodeSlc.cpp:476-494.
cf sinc2d_chip(const cf* chip, int rows, int cols, double x, double y) {
    const SincTable& T = sinc_table();
    const int half = SINC_LEN / 2;
    const int ix = (int)std::floor(x), iy = (int)std::floor(y);
    const double fx = x - ix, fy = y - iy;
    cf ret{0.f, 0.f};
    if ((ix < (half - 1)) || (ix > (cols - half - 1))) return ret;
    if ((iy < (half - 1)) || (iy > (rows - half - 1))) return ret;
    const int xx = ix + half, yy = iy + half;
    int ifracx = std::min(std::max(0, int(fx * SINC_SUB)), SINC_SUB - 1);
    int ifracy = std::min(std::max(0, int(fy * SINC_SUB)), SINC_SUB - 1);
    for (int i = 0; i < SINC_LEN; i++) {
        for (int j = 0; j < SINC_LEN; j++) {
            cf a = chip[(yy - i) * cols + (xx - j)];
            cf ky{(float)T.k[(size_t)ifracy * SINC_LEN + i], 0.f};
            cf kx{(float)T.k[(size_t)ifracx * SINC_LEN + j], 0.f};
            cf term = cmul(cmul(a, ky), kx);
            ret.re = ret.re + term.re;
            ret.im = ret.im + term.im;
        }
    }
    return ret;
}

// U = double flavour, used only by the interpolator known-answer test.
double sinc2d_double(const double* z, int rows, int cols, double x, double y) {
    const SincTable& T = sinc_table();
    const int half = SINC_LEN / 2;
    const int ix = (int)std::floor(x), iy = (int)std::floor(y);
    const double fx = x - ix, fy = y - iy;
    if ((ix < (half - 1)) || (ix > (cols - half - 1))) return 0.0;
    if ((iy < (half - 1)) || (iy > (rows - half - 1))) return 0.0;
    const int xx = ix + half, yy = iy + half;
    int ifracx = std::min(std::max(0, int(fx * SINC_SUB)), SINC_SUB - 1);
    int ifracy = std::min(std::max(0, int(fy * SINC_SUB)), SINC_SUB - 1);
    double ret = 0.0;
    for (int i = 0; i < SINC_LEN; i++)
        for (int j = 0; j < SINC_LEN; j++)
            ret += z[(size_t)(yy - i) * cols + (xx - j)] * T.k[(size_t)ifracy * SINC_LEN + i] *
                   T.k[(size_t)ifracx * SINC_LEN + j];
    return ret;
}

// ---------------------------------------------------------------- DEM
struct DEM {
    bool have_raster = false;
    double ref_height = 0.0;
    int epsg = 4326;
    Proj proj;
    double xstart = 0, ystart = 0, deltax = 0, deltay = 0;
    long width = 0, length = 0;
    std::vector<float> dem;
};

// geometry/DEMInterpolator.cpp:29-455 (loadDEM with bounding box)
int load_dem(DEM& d, const orc_dem_raster* r, double min_x, double max_x, double min_y, double max_y) {
    const double delta_y = r->gt[5];
    const double delta_x = r->gt[1];
    if (delta_x < 0) return 1;
    const double dem_y0 = r->gt[3];
    double dem_x0 = r->gt[0];
    int epsgcode = r->epsg;
    d.epsg = epsgcode;
    d.proj.init(epsgcode);
    if (epsgcode == 4326) {
        if (max_x - min_x > 360 + 2 * delta_x) max_x = min_x + 360 + delta_x;
        if (min_x < -180 - delta_x || max_x < -180 - delta_x || max_x > 360 + delta_x) {
            double n_wraps = std::floor(max_x / 360);
            min_x -= n_wraps * 360;
            max_x -= n_wraps * 360;
        }
        if (min_x < -180 - delta_x || max_x < -180 - delta_x) { min_x += 360; max_x += 360; }
        if (min_x > 0 && max_x < 0) max_x += 360;
        if (dem_x0 > 360 + delta_x || dem_x0 < -180 - delta_x) dem_x0 = std::fmod(dem_x0, 360);
    }
    const double dem_yf = dem_y0 + r->length * delta_y;
    const double dem_xf = dem_x0 + r->width * delta_x;
    if (epsgcode == 4326 && min_x < dem_xf - 360 - delta_x) { min_x += 360; max_x += 360; }
    else if (epsgcode == 4326 && min_x > 180 && max_x > dem_x0 + 360 + delta_x) { min_x -= 360; max_x -= 360; }
    bool disc = (epsgcode == 4326) && (min_x <= dem_xf) && (dem_xf < max_x) &&
                (min_x <= dem_x0 + 360) && (dem_x0 + 360 < max_x);
    if (min_x < dem_x0) min_x = dem_x0;
    if (max_x > dem_xf && !disc) max_x = dem_xf;
    if (min_y < dem_yf) min_y = dem_yf;
    if (max_y > dem_y0) max_y = dem_y0;
    long min_x_idx = (long)std::floor((min_x - dem_x0) / delta_x);
    long max_x_idx = (long)std::ceil((max_x - dem_x0) / delta_x);
    long min_y_idx = (long)std::floor((max_y - dem_y0) / delta_y);
    long max_y_idx = (long)std::ceil((min_y - dem_y0) / delta_y);
    d.xstart = dem_x0 + (0.5 + min_x_idx) * delta_x;
    d.ystart = dem_y0 + (0.5 + min_y_idx) * delta_y;
    d.deltax = delta_x;
    d.deltay = delta_y;
    long width = max_x_idx - min_x_idx;
    long length = max_y_idx - min_y_idx;
    if (!disc && min_x_idx + width > r->width) { width = r->width - min_x_idx; max_x_idx = min_x_idx + width; }
    if (!disc && min_y_idx + length > r->length) { length = r->length - min_y_idx; max_y_idx = min_y_idx + length; }
    if (width <= 0 || length <= 0) return 2;
    d.width = width; d.length = length;
    d.dem.assign((size_t)width * length, 0.f);
    // GDAL getBlock of a window that is partly outside the raster is an
    // error in the reference; here the window is inside by construction
    // except for negative offsets, which GDAL would also reject.
    if (min_x_idx < 0 || min_y_idx < 0) return 3;
    if (!disc) {
        for (long i = 0; i < length; ++i)
            std::memcpy(&d.dem[(size_t)i * width], &r->data[(size_t)(min_y_idx + i) * r->width + min_x_idx],
                        sizeof(float) * width);
    } else {
        std::fill(d.dem.begin(), d.dem.end(), std::numeric_limits<float>::quiet_NaN());
        const long wl = r->width - min_x_idx;
        for (long i = 0; i < length && wl > 0; ++i)
            for (long j = 0; j < wl; ++j)
                d.dem[(size_t)i * width + j] = r->data[(size_t)(min_y_idx + i) * r->width + min_x_idx + j];
        const double ideal = (r->width - 360.0 / delta_x);
        const long wnext = std::lround(ideal);
        if (std::abs(ideal - wnext) > 1e-5) return 4;
        const long x0r = std::max(0L, wnext);
        const long x1r = std::min((long)(r->width - 1), (long)std::ceil((max_x - 360 - dem_x0) / delta_x));
        const long wr = x1r - x0r;
        if (wr > 1) {
            for (long i = 0; i < length; ++i)
                for (long j = 0; j < wr; ++j) {
                    const long dj = (long)((x0r + j) + 360.0 / delta_x - min_x_idx);
                    if (dj > width - 1) continue;
                    d.dem[(size_t)i * width + dj] = r->data[(size_t)(min_y_idx + i) * r->width + x0r + j];
                }
        }
    }
    d.have_raster = true;
    return 0;
}

// geometry/loadDem.cpp:22-133 (DEMRasterToInterpolator, BIQUINTIC)
int dem_raster_to_interp(DEM& d, const orc_dem_raster* r, const orc_geo_grid* g, int lineStart,
                         int blockLength, int blockWidth, int margin) {
    d = DEM();
    d.ref_height = 0.0;
    double minX = std::numeric_limits<double>::max();
    double maxX = std::numeric_limits<double>::lowest();
    double minY = std::numeric_limits<double>::max();
    double maxY = std::numeric_limits<double>::lowest();
    if (r->epsg != g->epsg) {
        Proj proj, demproj;
        if (!proj.init(g->epsg) || !demproj.init(r->epsg)) return fail("unsupported EPSG");
        const int askip = std::max(static_cast<int>(blockLength / 10.), 1);
        const int rskip = std::max(static_cast<int>(blockWidth / 10.), 1);
        std::vector<int> lineInd, pixInd;
        for (int j = 0; j < blockWidth; j += rskip) { lineInd.push_back(0); pixInd.push_back(j); }
        for (int i = 0; i < blockLength; i += askip) { lineInd.push_back(i); pixInd.push_back(blockWidth); }
        for (int j = blockWidth; j > 0; j -= rskip) { lineInd.push_back(blockLength - 1); pixInd.push_back(j); }
        for (int i = blockLength; i > 0; i -= askip) { lineInd.push_back(i); pixInd.push_back(0); }
        for (size_t i = 0; i < lineInd.size(); i++) {
            V3 outpt{g->start_x + g->spacing_x * pixInd[i],
                     g->start_y + g->spacing_y * (lineStart + lineInd[i]), 0.0};
            V3 tmp, dempt;
            if (proj.inverse(outpt, tmp) != 0 || demproj.forward(tmp, dempt) != 0)
                return fail("projection transformation between geogrid and DEM failed");
            minX = std::min(minX, dempt.x); maxX = std::max(maxX, dempt.x);
            minY = std::min(minY, dempt.y); maxY = std::max(maxY, dempt.y);
        }
    } else {
        maxY = g->start_y + g->spacing_y * lineStart;
        minY = g->start_y + g->spacing_y * (lineStart + blockLength - 1);
        minX = g->start_x;
        maxX = g->start_x + g->spacing_x * (blockWidth - 1);
    }
    minX -= margin * r->gt[1];
    maxX += margin * r->gt[1];
    minY -= margin * std::abs(r->gt[5]);
    maxY += margin * std::abs(r->gt[5]);
    int st = load_dem(d, r, minX, maxX, minY, maxY);
    if (st != 0) d.have_raster = false;   // interpolation then returns refHeight
    d.epsg = r->epsg;
    d.proj.init(r->epsg);
    return 0;
}

// geometry/DEMInterpolator.cpp:617-659
double dem_interp_xy(const DEM& d, double x, double y) {
    double value = d.ref_height;
    if (!d.have_raster) return value;
    if (d.epsg == 4326 && (x > 360 || x < -360)) x = std::fmod(x, 360);
    if (d.epsg == 4326 && x < -180) x += 360;
    if (d.epsg == 4326 && x - 360 >= d.xstart) {
        x -= 360;
    } else if (d.epsg == 4326 && x < d.xstart && x + 360 >= d.xstart) {
        x += 360;
    } else if (x < d.xstart) {
        return d.ref_height;
    }
    const double row = (y - d.ystart) / d.deltay;
    const double col = (x - d.xstart) / d.deltax;
    const int irow = int(std::floor(row));
    const int icol = int(std::floor(col));
    if (irow < 2 || irow >= int(d.length - 1)) return d.ref_height;
    if (icol < 2 || icol >= int(d.width - 1)) return d.ref_height;
    return (double)spline2d<float>(d.dem.data(), (int)d.length, (int)d.width, col, row);
}

// geometry/DEMInterpolator.cpp:593-611
double dem_interp_lonlat(const DEM& d, double lon, double lat) {
    if (!d.have_raster) return d.ref_height;
    V3 xyz{0, 0, 0};
    d.proj.forward({lon, lat, 0.0}, xyz);
    return dem_interp_xy(d, xyz.x, xyz.y);
}

// cuda/core/gpuSpline2dInterpolator.cu:85-101 for T = float: the double
// literals promote parts of each expression to double.
void init_spline_gpu(const float* Y, int n, float* R, float* Q) {
    Q[0] = 0.0f;
    R[0] = 0.0f;
    for (int i = 1; i < n - 1; ++i) {
        const double p = 1.0 / (0.5 * Q[i - 1] + 2.0);
        Q[i] = (float)(-0.5 * p);
        R[i] = (float)((3 * (Y[i + 1] - 2 * Y[i] + Y[i - 1]) - 0.5 * R[i - 1]) * p);
    }
    R[n - 1] = 0.0f;
    for (int i = (n - 2); i > 0; --i) R[i] = Q[i] * R[i + 1] + R[i];
}

// cuda/core/gpuSpline2dInterpolator.cu:103-117
float spline_gpu(double x, const float* Y, int n, const float* R) {
    if (x < 1.0) {
        return (float)(Y[0] + (x - 1.0) * (Y[1] - Y[0] - (R[1] / 6.0)));
    } else if (x > n) {
        return (float)(Y[n - 1] + ((x - n) * (Y[n - 1] - Y[n - 2] + (R[n - 2] / 6.))));
    } else {
        int j = int(std::floor(x));
        double xx = x - j;
        double t0 = Y[j] - Y[j - 1] - (R[j - 1] / 3.0) - (R[j] / 6.0);
        double t1 = xx * ((R[j - 1] / 2.0) + (xx * ((R[j] - R[j - 1]) / 6)));
        return (float)(Y[j - 1] + (xx * (t0 + t1)));
    }
}

// cuda/core/gpuSpline2dInterpolator.cu:119-145 (order 6; MAX_ORDER arrays
// zero-initialised as there)
float spline2d_gpu(const float* z, int ny, int nx, double x, double y) {
    const int order = 6;
    int i0 = (int)y, j0 = (int)x;
    i0 = i0 - (order / 2) + 1;
    j0 = j0 - (order / 2) + 1;
    float A[20] = {0}, R[20] = {0}, Q[20] = {0}, HC[20] = {0};
    for (int i = 0; i < order; ++i) {
        const int indi = std::min(std::max(i0 + i, 0), ny - 2);
        for (int j = 0; j < order; ++j) {
            const int indj = std::min(std::max(j0 + j, 0), nx - 2);
            A[j] = z[(size_t)(indi + 1) * nx + indj + 1];
        }
        init_spline_gpu(A, order, R, Q);
        HC[i] = spline_gpu(x - j0, A, order, R);
    }
    init_spline_gpu(HC, order, R, Q);
    return spline_gpu(y - i0, HC, order, R);
}

// cuda/geometry/gpuDEMInterpolator.cu:149-204: projection forward, no +-360
// wrap, float result
float dem_interp_lonlat_gpu(const DEM& d, double lon, double lat) {
    float value = (float)d.ref_height;
    if (!d.have_raster) return value;
    V3 xyz{0, 0, 0};
    d.proj.forward({lon, lat, 0.0}, xyz);
    const double row = (xyz.y - d.ystart) / d.deltay;
    const double col = (xyz.x - d.xstart) / d.deltax;
    const int irow = int(std::floor(row));
    const int icol = int(std::floor(col));
    if (irow < 2 || irow >= int(d.length - 1)) return (float)d.ref_height;
    if (icol < 2 || icol >= int(d.width - 1)) return (float)d.ref_height;
    return spline2d_gpu(d.dem.data(), (int)d.length, (int)d.width, col, row);
}

// ---------------------------------------------------------------- geo2rdr
enum { G_OK = 0, G_OOB = 1, G_LOOK = 2, G_NOCONV = 3 };

// geometry/detail/Geo2Rdr.icc:11-48
int doppler_aztime_diff(double* dt, double t, double r, V3 rvec, V3 vel, const orc_lut2d* dop,
                        double wvl, double dr) {
    if (dop->bounds_error) {
        if (!(lut_contains(dop, t, r) && lut_contains(dop, t, r + dr))) return G_OOB;
    }
    const double dopfact = dot(rvec, vel);
    const double fdop = 0.5 * wvl * lut_eval(dop, t, r);
    const double fdopder = (0.5 * wvl * lut_eval(dop, t, r + dr) - fdop) / dr;
    const double fn = dopfact - fdop * r;
    const double c1 = -dot(vel, vel);
    const double c2 = (fdop / r) + fdopder;
    const double fnprime = c1 + c2 * dopfact;
    *dt = fn / fnprime;
    return G_OK;
}

// geometry/detail/Geo2Rdr.icc:50-112
int update_aztime(double* t, const orc_orbit* o, V3 xyz, int side) {
    const int num = 15;
    const double tstart = o->t0, tend = orb_time(o, o->n - 1);
    const double dt = (tend - tstart) / (num - 1);
    double r_closest = 1e16, t_closest = -1000.;
    for (int k = 0; k < num; ++k) {
        const double tt = tstart + k * dt;
        if (tt < tstart || tt > tend) continue;
        V3 pos, vel;
        orbit_interp(o, tt, &pos, &vel);
        const V3 rvec = sub(xyz, pos);
        if (k == 0) {
            if ((side == -1) != (dot(cross(rvec, vel), pos) > 0.)) return G_LOOK;
        }
        const double r = norm(rvec);
        if (r < r_closest) { r_closest = r; t_closest = tt; }
    }
    *t = (t_closest < 0.) ? 0.5 * (tstart + tend) : t_closest;
    return G_OK;
}

// geometry/detail/Geo2Rdr.icc:114-179
int geo2rdr_detail(double* t, double* r, V3 llh, double a, double e2, const orc_orbit* o,
                   const orc_lut2d* dop, double wvl, int side, double t0, double thr, int maxiter,
                   double dr, int* iters = nullptr) {
    const V3 xyz = lonlat_to_xyz(a, e2, llh);
    if (t0 >= o->t0 && t0 <= orb_time(o, o->n - 1)) {
        *t = t0;
    } else {
        int st = update_aztime(t, o, xyz, side);
        if (st != G_OK) return st;
    }
    double dt = 0.0;
    for (int i = 0; i < maxiter; ++i) {
        *t -= dt;
        V3 pos, vel;
        orbit_interp(o, *t, &pos, &vel);
        const V3 rvec = sub(xyz, pos);
        *r = norm(rvec);
        if (i == 0) {
            if ((side == -1) != (dot(cross(rvec, vel), pos) > 0.)) return G_LOOK;
        }
        int st = doppler_aztime_diff(&dt, *t, *r, rvec, vel, dop, wvl, dr);
        if (st != G_OK) return st;
        if (iters) *iters = i + 1;
        if (std::abs(dt) < thr) return G_OK;
    }
    return G_NOCONV;
}

// ---------------------------------------------------------------- radar grid
inline double rg_sensing_stop(const orc_radar_grid& g) { return g.sensing_start + (g.length - 1.0) / g.prf; }
inline double rg_ending_range(const orc_radar_grid& g) { return g.starting_range + (g.width - 1.0) * g.range_pixel_spacing; }
inline double rg_sensing_mid(const orc_radar_grid& g) { return 0.5 * (g.sensing_start + rg_sensing_stop(g)); }
// product/RadarGridParameters.cpp:27-35
bool rg_contains(const orc_radar_grid& g, double az, double sr) {
    const double half_az = (1.0 / g.prf) / 2;
    const double half_rg = g.range_pixel_spacing / 2;
    return az >= g.sensing_start - half_az && sr >= g.starting_range - half_rg &&
           az <= rg_sensing_stop(g) + half_az && sr <= rg_ending_range(g) + half_rg;
}

// product/SubSwaths.cpp:58-96
int subswath_of(const orc_subswaths* s, int az, int rg) {
    if (rg < 0 || rg >= s->width || az < 0 || az >= s->length) return 0;
    if (s->n == 0) return 1;
    for (int k = 1; k <= s->n; ++k) {
        const int32_t* v = s->valid + (size_t)(k - 1) * s->length * 2;
        const int start = v[(size_t)az * 2], stop = v[(size_t)az * 2 + 1];
        if (rg >= start && rg < stop) return k;
    }
    return 0;
}

// geocode/geocodeSlc.cpp:548-580
int validate_slice(const orc_radar_grid& full, const orc_radar_grid& s) {
    if (s.sensing_start < full.sensing_start) return fail("sliced grid sensing start < full grid sensing start");
    if (rg_sensing_stop(s) > rg_sensing_stop(full)) return fail("sliced grid sensing stop < full grid sensing stop");
    if (s.starting_range < full.starting_range) return fail("sliced grid staring range < full grid staring range");
    if (rg_ending_range(s) > rg_ending_range(full)) return fail("sliced grid ending range < full grid ending range");
    if (s.look_side != full.look_side) return fail("sliced grid look side != full grid look side");
    if (s.wavelength != full.wavelength) return fail("sliced grid wavelength != full grid wavelength");
    return 0;
}

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ================================================================ geocode
namespace {

// Radar bounding box of a block's valid pixels (geocodeSlc.cpp:79-85, 210-221)
struct Bbox {
    int az0, az1, rg0, rg1;
};

// computeGeogridRadarIndicesAndMask (geocodeSlc.cpp:55-228) over geogrid
// lines [line0, line0 + nlines) with the block's DEM interpolator.  Indices,
// uncorrected slant range, mask and iteration counts are block-relative
// (row blockLine = line - line0).  Returns 1 if a projection inverse failed.
int radar_indices(const orc_geocode_args* a, const Proj& proj, const DEM& dem, long line0, long nlines,
                  std::vector<double>& rgIdx, std::vector<double>& azIdx, std::vector<double>& uncorr,
                  uint8_t* mask, const orc_subswaths* subswaths, uint8_t* out_niter, Bbox& bb) {
    const orc_radar_grid& rg = a->radar_grid;
    const orc_radar_grid& srg = a->sliced_radar_grid;
    const orc_geo_grid& gg = a->geo_grid;
    const size_t W = gg.width;
    const bool useCorr = a->flatten_with_corrected_srange != 0;
    const int chipHalf = SINC_ONE / 2;
    int az0 = (int)rg.length - 1, az1 = 0, rg0 = (int)rg.width - 1, rg1 = 0;
    int proj_fail = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(min : az0, rg0) reduction(max : az1, rg1)
    for (long blockLine = 0; blockLine < nlines; ++blockLine) {
        const long line = line0 + blockLine;
        for (size_t pixel = 0; pixel < W; ++pixel) {
            const size_t k = (size_t)blockLine * W + pixel;
            double y = gg.start_y + gg.spacing_y * (line + 0.5);
            double x = gg.start_x + gg.spacing_x * (pixel + 0.5);
            double aztime = rg_sensing_mid(rg), srange = 0.0;
            V3 llh;
            if (proj.inverse({x, y, 0.0}, llh) != 0) {
#pragma omp atomic write
                proj_fail = 1;
                continue;
            }
            llh.z = dem_interp_lonlat(dem, llh.x, llh.y);
            int niter = 0;
            int st = geo2rdr_detail(&aztime, &srange, llh, a->ell_a, a->ell_e2, &a->orbit,
                                    &a->image_grid_doppler, rg.wavelength, rg.look_side, aztime,
                                    a->threshold_geo2rdr, a->numiter_geo2rdr, 1.0e-8, &niter);
            if (out_niter) out_niter[k] = st == G_OK ? (uint8_t)std::min(niter, 255) : 0;
            if (st != G_OK) continue;
            if (!useCorr) uncorr[k] = srange;
            if (lut_contains(&a->az_time_correction, aztime, srange))
                aztime += lut_eval(&a->az_time_correction, aztime, srange);
            if (lut_contains(&a->srange_correction, aztime, srange))
                srange += lut_eval(&a->srange_correction, aztime, srange);
            if (!rg_contains(srg, aztime, srange) || !lut_contains(&a->native_doppler, aztime, srange))
                continue;
            double azc = (aztime - rg.sensing_start) * rg.prf;
            double rgc = (srange - rg.starting_range) / rg.range_pixel_spacing;
            const int intAz = (int)std::floor(azc);
            const int intRg = (int)std::floor(rgc);
            bool corners = true;
            if ((intRg < chipHalf) || (intRg >= (rg.width - chipHalf)) || (intAz < chipHalf) ||
                (intAz >= (rg.length - chipHalf)))
                corners = false;
            if (subswaths && mask) {
                unsigned char m = (unsigned char)subswath_of(subswaths, intAz, intRg);
                if (m != 0) {
                    const int ext[2] = {-chipHalf, chipHalf};
                    for (int ai = 0; ai < 2; ++ai)
                        for (int ri = 0; ri < 2; ++ri)
                            if (subswath_of(subswaths, intAz + ext[ai], intRg + ext[ri]) == 0) { m = 0; break; }
                }
                mask[k] = m;
            } else if (corners && mask) {
                mask[k] = 1;
            }
            az0 = std::min(az0, (int)std::floor(azc));
            az1 = std::max(az1, (int)(std::ceil(azc) - 1));
            rg0 = std::min(rg0, (int)std::floor(rgc));
            rg1 = std::max(rg1, (int)(std::ceil(rgc) - 1));
            rgIdx[k] = rgc;
            azIdx[k] = azc;
        }
    }
    bb = Bbox{az0, az1, rg0, rg1};
    return proj_fail;
}

// carrierPhaseDeramp (geocodeSlc.cpp:240-274) of an inL x inW radar block
// whose first sample is line azFirst, sample rgFirst of the radar grid
void deramp_block(const orc_geocode_args* a, cf* rdr, long inL, long inW, size_t azFirst, size_t rgFirst) {
    const orc_radar_grid& rg = a->radar_grid;
#pragma omp parallel for
    for (long ii = 0; ii < inL * inW; ++ii) {
        size_t i = ii / inW, j = ii % inW;
        const size_t i_az = i + azFirst;
        const double az = rg.sensing_start + i_az / rg.prf;
        const size_t j_rg = j + rgFirst;
        const double r = rg.starting_range + j_rg * rg.range_pixel_spacing;
        const float carrierPhase = azrg_eval(&a->rg_carrier, az, r) + azrg_eval(&a->az_carrier, az, r);
        const cf c{std::cos(carrierPhase), -std::sin(carrierPhase)};
        rdr[ii] = cmul(rdr[ii], c);
    }
}

// interpolate (geocodeSlc.cpp:409-511): N geo pixels from the deramped block
void interpolate_block(const orc_geocode_args* a, const cf* rdr, long inL, long inW, size_t azFirst,
                       size_t rgFirst, const double* rgIdx, const double* azIdx, size_t N, cf* geo) {
    const orc_radar_grid& rg = a->radar_grid;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long ii = 0; ii < (long)N; ++ii) {
        const double uRg = rgIdx[ii], uAz = azIdx[ii];
        if (std::isnan(uRg) || std::isnan(uAz)) continue;
        double RgIndex = uRg - (double)rgFirst;
        double AzIndex = uAz - (double)azFirst;
        const int intRg = (int)RgIndex, intAz = (int)AzIndex;
        const double fracRg = RgIndex - intRg, fracAz = AzIndex - intAz;
        if ((intRg < SINC_HALF) || (intRg >= (inW - SINC_HALF))) continue;
        if ((intAz < SINC_HALF) || (intAz >= (inL - SINC_HALF))) continue;
        const double rng = rg.starting_range + uRg * rg.range_pixel_spacing;
        const double az = rg.sensing_start + uAz / rg.prf;
        if (!lut_contains(&a->native_doppler, az, rng)) continue;
        const double doppFreq = lut_eval(&a->native_doppler, az, rng) * 2 * M_PI / rg.prf;
        cf chip[SINC_ONE * SINC_ONE];
        for (int r9 = 0; r9 < SINC_ONE; ++r9) {
            const int chipRow = intAz + r9 - SINC_HALF;
            const double doppPhase = doppFreq * (r9 - SINC_HALF);
            const cf dv{(float)std::cos(doppPhase), (float)-std::sin(doppPhase)};
            for (int c9 = 0; c9 < SINC_ONE; ++c9) {
                const int chipCol = intRg + c9 - SINC_HALF;
                chip[r9 * SINC_ONE + c9] = cmul(rdr[(size_t)chipRow * inW + chipCol], dv);
            }
        }
        const cf cval = sinc2d_chip(chip, SINC_ONE, SINC_ONE, SINC_HALF + fracRg, SINC_HALF + fracAz);
        const double back = doppFreq * fracAz;
        const cf bv{(float)std::cos(back), (float)std::sin(back)};
        geo[ii] = cmul(cval, bv);
    }
}

// carrierPhaseRerampAndFlatten (geocodeSlc.cpp:298-394)
void reramp_block(const orc_geocode_args* a, long inL, long inW, size_t azFirst, size_t rgFirst,
                  const double* rgIdx, const double* azIdx, const double* uncorr, size_t N, cf* geo,
                  double* carrier_phase, double* flatten_phase) {
    const orc_radar_grid& rg = a->radar_grid;
    const bool useCorr = a->flatten_with_corrected_srange != 0;
    const int chipHalf = SINC_ONE / 2;
#pragma omp parallel for schedule(dynamic, 4096)
    for (long ii = 0; ii < (long)N; ++ii) {
        const double uRg = rgIdx[ii], uAz = azIdx[ii];
        if (std::isnan(uRg) || std::isnan(uAz)) continue;
        const double RgIndex = uRg - (double)rgFirst, AzIndex = uAz - (double)azFirst;
        const int intRg = (int)RgIndex, intAz = (int)AzIndex;
        if ((intRg < chipHalf) || (intRg >= (inW - chipHalf))) continue;
        if ((intAz < chipHalf) || (intAz >= (inL - chipHalf))) continue;
        const double rng = rg.starting_range + uRg * rg.range_pixel_spacing;
        const double az = rg.sensing_start + uAz / rg.prf;
        if (!lut_contains(&a->native_doppler, az, rng)) continue;
        const double carrierPhase = azrg_eval(&a->rg_carrier, az, rng) + azrg_eval(&a->az_carrier, az, rng);
        const double sRngFlatten = useCorr ? rng : uncorr[ii];
        const double flattenPhase = 4.0 * (M_PI / rg.wavelength) * sRngFlatten;
        double totalPhase = 0.0;
        if (a->reramp) totalPhase += carrierPhase;
        if (a->flatten) totalPhase += flattenPhase;
        if (carrier_phase) carrier_phase[ii] = carrierPhase;
        if (flatten_phase) flatten_phase[ii] = flattenPhase;
        const cf c{(float)std::cos(totalPhase), (float)std::sin(totalPhase)};
        geo[ii] = cmul(geo[ii], c);
    }
}

}  // namespace

// Array mode (geocodeSlc.cpp:831-968): the whole geogrid is one block with
// one DEM window; the caller's radar blocks start at (first_azimuth_line,
// first_range_sample).
extern "C" int orc_geocode_slc(orc_geocode_args* a) {
    g_err.clear();
    const orc_radar_grid& rg = a->radar_grid;
    const orc_radar_grid& srg = a->sliced_radar_grid;
    const orc_geo_grid& gg = a->geo_grid;
    const size_t L = gg.length, W = gg.width;
    const size_t N = L * W;
    if (a->n_blocks < 1) return fail("number of geoDataBlocks != number of rdrDataBlocks");
#ifdef _OPENMP
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
#endif
    // geocodeSlc.cpp:873-877
    for (int b = 0; b < a->n_blocks; ++b)
        for (size_t k = 0; k < N; ++k) { a->geo_blocks[b][2*k] = a->invalid_re; a->geo_blocks[b][2*k+1] = a->invalid_im; }
    if (a->mask) std::memset(a->mask, 255, N);
    if (validate_slice(rg, srg)) return 1;
    Proj proj;
    if (!proj.init(gg.epsg)) return fail("Unknown EPSG code (in factory): " + std::to_string(gg.epsg));
    (void)sinc_table();
    DEM dem;
    if (dem_raster_to_interp(dem, &a->dem, &gg, 0, (int)L, (int)W, a->dem_margin)) return 1;

    std::vector<double> rgIdx(N, NaN), azIdx(N, NaN);
    std::vector<double> uncorr;
    const bool useCorr = a->flatten_with_corrected_srange != 0;
    if (!useCorr) uncorr.assign(N, (double)a->invalid_re);

    double t_start = now();
    Bbox bb;
    if (radar_indices(a, proj, dem, 0, (long)L, rgIdx, azIdx, uncorr, a->mask, a->subswaths, a->out_niter, bb))
        return fail("Inverse projection transformation failed");
    a->phase_seconds[0] = now() - t_start;
    a->phase_seconds[1] = a->phase_seconds[2] = a->phase_seconds[3] = 0.0;

    if (a->out_az_index) std::memcpy(a->out_az_index, azIdx.data(), N * sizeof(double));
    if (a->out_rg_index) std::memcpy(a->out_rg_index, rgIdx.data(), N * sizeof(double));
    if (a->out_uncorrected_srange && !useCorr) std::memcpy(a->out_uncorrected_srange, uncorr.data(), N * sizeof(double));

    const long inL = a->rdr_length, inW = a->rdr_width;
    const size_t azFirst = a->first_azimuth_line, rgFirst = a->first_range_sample;
    for (int b = 0; b < a->n_blocks; ++b) {
        cf* rdr = reinterpret_cast<cf*>(a->rdr_blocks[b]);
        cf* geo = reinterpret_cast<cf*>(a->geo_blocks[b]);
        t_start = now();
        deramp_block(a, rdr, inL, inW, azFirst, rgFirst);
        a->phase_seconds[1] += now() - t_start;
        t_start = now();
        interpolate_block(a, rdr, inL, inW, azFirst, rgFirst, rgIdx.data(), azIdx.data(), N, geo);
        a->phase_seconds[2] += now() - t_start;
        t_start = now();
        reramp_block(a, inL, inW, azFirst, rgFirst, rgIdx.data(), azIdx.data(), useCorr ? nullptr : uncorr.data(), N,
                     geo, a->carrier_phase, a->flatten_phase);
        a->phase_seconds[3] += now() - t_start;
    }
    return 0;
}

// Raster mode (geocodeSlc.cpp:605-828).  rdr_blocks are the input raster's
// bands over the whole radar grid (rdr_length x rdr_width = the grid), read
// only; geo_blocks, carrier_phase and flatten_phase the output rasters over
// the whole geogrid.  Per block of lines_per_block geogrid lines: the
// block's own DEM window, the radar indices and their bounding box, the box
// widened by 5 samples and clamped to the radar grid, invalid fill (and
// invalid_re in the phase rasters), then per band the box read out of the
// input raster, deramped, interpolated and reramped.  mask, the offsets and
// subswaths are not used (the reference's raster mode has none).
extern "C" int orc_geocode_slc_raster(orc_geocode_args* a, int32_t lines_per_block) {
    g_err.clear();
    const orc_radar_grid& rg = a->radar_grid;
    const orc_geo_grid& gg = a->geo_grid;
    const long W = gg.width, Lg = gg.length;
    if (lines_per_block < 1) return fail("lines_per_block must be positive");
    if (a->n_blocks < 1) return fail("number of input and output bands differ");
    if (a->rdr_length != rg.length || a->rdr_width != rg.width)
        return fail("input raster shape differs from the radar grid");
#ifdef _OPENMP
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
#endif
    if (validate_slice(rg, a->sliced_radar_grid)) return 1;
    Proj proj;
    if (!proj.init(gg.epsg)) return fail("Unknown EPSG code (in factory): " + std::to_string(gg.epsg));
    (void)sinc_table();
    const bool useCorr = a->flatten_with_corrected_srange != 0;
    const long nBlocks = (Lg + lines_per_block - 1) / lines_per_block;
    for (long block = 0; block < nBlocks; ++block) {
        const long lineStart = block * lines_per_block;
        const long geoBlockLength = (block == nBlocks - 1) ? Lg - lineStart : lines_per_block;
        const size_t n = (size_t)geoBlockLength * W;
        const size_t off = (size_t)lineStart * W;
        DEM dem;
        if (dem_raster_to_interp(dem, &a->dem, &gg, (int)lineStart, (int)geoBlockLength, (int)W, a->dem_margin))
            return 1;
        std::vector<double> rgIdx(n, NaN), azIdx(n, NaN), uncorr;
        if (!useCorr) uncorr.assign(n, (double)a->invalid_re);
        std::vector<uint8_t> dummy_mask(n, 0);
        Bbox bb;
        if (radar_indices(a, proj, dem, lineStart, geoBlockLength, rgIdx, azIdx, uncorr, dummy_mask.data(), nullptr,
                          nullptr, bb))
            return fail("Inverse projection transformation failed");
        if (a->out_az_index) std::memcpy(a->out_az_index + off, azIdx.data(), n * sizeof(double));
        if (a->out_rg_index) std::memcpy(a->out_rg_index + off, rgIdx.data(), n * sizeof(double));
        // invalid fill of the block and its phase rasters
        for (int b = 0; b < a->n_blocks; ++b)
            for (size_t k = 0; k < n; ++k) {
                a->geo_blocks[b][2 * (off + k)] = a->invalid_re;
                a->geo_blocks[b][2 * (off + k) + 1] = a->invalid_im;
            }
        if (a->carrier_phase) std::fill(a->carrier_phase + off, a->carrier_phase + off + n, (double)a->invalid_re);
        if (a->flatten_phase) std::fill(a->flatten_phase + off, a->flatten_phase + off + n, (double)a->invalid_re);
        // geocodeSlc.cpp:740-750: interpolation margin, clamped to the radar grid
        const int interp_margin = 5;
        const int az0 = std::max(bb.az0 - interp_margin, 0);
        const int rg0 = std::max(bb.rg0 - interp_margin, 0);
        const int az1 = std::min(bb.az1 + interp_margin, (int)(rg.length - 1));
        const int rg1 = std::min(bb.rg1 + interp_margin, (int)(rg.width - 1));
        if (az0 > az1 || rg0 > rg1) continue;       // :752-770, no valid pixels
        const long inL = az1 - az0 + 1, inW = rg1 - rg0 + 1;
        std::vector<cf> rdr((size_t)inL * inW);
        for (int b = 0; b < a->n_blocks; ++b) {
            const cf* band = reinterpret_cast<const cf*>(a->rdr_blocks[b]);
            for (long i = 0; i < inL; ++i)
                std::memcpy(&rdr[(size_t)i * inW], band + (size_t)(az0 + i) * rg.width + rg0, inW * sizeof(cf));
            cf* geo = reinterpret_cast<cf*>(a->geo_blocks[b]) + off;
            deramp_block(a, rdr.data(), inL, inW, (size_t)az0, (size_t)rg0);
            interpolate_block(a, rdr.data(), inL, inW, (size_t)az0, (size_t)rg0, rgIdx.data(), azIdx.data(), n, geo);
            // the phase rasters are written for every band, with the same values
            reramp_block(a, inL, inW, (size_t)az0, (size_t)rg0, rgIdx.data(), azIdx.data(),
                         useCorr ? nullptr : uncorr.data(), n, geo, a->carrier_phase ? a->carrier_phase + off : nullptr,
                         a->flatten_phase ? a->flatten_phase + off : nullptr);
        }
    }
    return 0;
}

extern "C" const char* orc_last_error(void) { return g_err.c_str(); }

// ================================================================ raster geocode
namespace {

// cuda/product/SubSwaths.h:177-205 (ViewSubSwaths::contains)
bool subswath_contains_gpu(const orc_subswaths* s, int az, int rg) {
    if (!s || s->n == 0) return true;
    if (az < 0 || az >= s->length || rg < 0 || rg >= s->width) return false;
    for (int k = 0; k < s->n; ++k) {
        const int32_t* v = s->valid + (size_t)k * s->length * 2;
        if (rg >= v[(size_t)az * 2] && rg < v[(size_t)az * 2 + 1]) return true;
    }
    return false;
}

}  // namespace

extern "C" int orc_geocode_rasters(orc_raster_args* a) {
    g_err.clear();
    const orc_radar_grid& rg = a->radar_grid;
    const orc_geo_grid& gg = a->geo_grid;
    if (a->lines_per_block < 1) return fail("lines_per_block must be positive");
    if (a->n_rasters < 1) return fail("number of input and output rasters not equal");
#ifdef _OPENMP
    if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
#endif
    Proj proj;
    if (!proj.init(gg.epsg)) return fail("unsupported geogrid EPSG");
    const long W = gg.width, Lg = gg.length;
    const long lpb = a->lines_per_block;
    const long n_blocks = (Lg + lpb - 1) / lpb;     // Geocode.cu:343
    const double t_mid = rg_sensing_mid(rg);
    const size_t rW = (size_t)rg.width, rL = (size_t)rg.length;
    for (long blk = 0; blk < n_blocks; ++blk) {
        // Geocode.cu:378-400: block extent
        const long line_start = blk * lpb;
        const long block_length = (blk == n_blocks - 1) ? Lg - line_start : lpb;
        const size_t n = (size_t)block_length * W;
        // Geocode.cu:402-407: the block's own DEM window
        DEM dem;
        if (dem_raster_to_interp(dem, &a->dem, &gg, (int)line_start, (int)block_length, (int)W, a->dem_margin))
            return 1;
        std::vector<double> rx(n), ry(n);
        std::vector<char> mask(n);
        // geoToRdrIndices, Geocode.cu:87-172
#pragma omp parallel for schedule(dynamic, 1024)
        for (long tid = 0; tid < (long)n; ++tid) {
            const long block_line = tid / W, pixel = tid % W;
            const long line = line_start + block_line;
            const V3 xyz{gg.start_x + gg.spacing_x * (0.5 + pixel), gg.start_y + gg.spacing_y * (0.5 + line), 0.0};
            V3 llh{0, 0, 0};
            // the CUDA kernel ignores the inverse's status; a failed inverse is masked here
            const bool proj_ok = proj.inverse(xyz, llh) == 0;
            llh.z = dem_interp_lonlat_gpu(dem, llh.x, llh.y);
            double srange = 0.0, aztime = t_mid;
            bool converged = false;
            if (proj_ok)
                converged = geo2rdr_detail(&aztime, &srange, llh, a->ell_a, a->ell_e2, &a->orbit, &a->doppler,
                                           rg.wavelength, rg.look_side, aztime, a->threshold, a->maxiter,
                                           a->delta_range) == G_OK;
            bool masked = false;
            if (converged) {
                if (lut_contains(&a->az_time_correction, aztime, srange))
                    aztime += lut_eval(&a->az_time_correction, aztime, srange);
                else
                    masked = true;
                if (lut_contains(&a->srange_correction, aztime, srange))
                    srange += lut_eval(&a->srange_correction, aztime, srange);
                else
                    masked = true;
                if (!lut_contains(&a->native_doppler, aztime, srange)) masked = true;
            }
            bool invalid = !converged || masked;
            double y = 0.0, x = 0.0;
            if (!invalid) {
                y = (aztime - rg.sensing_start) * rg.prf;
                x = (srange - rg.starting_range) / rg.range_pixel_spacing;
                const int y_int = (int)std::floor(y), x_int = (int)std::floor(x);
                if (!subswath_contains_gpu(a->subswaths, y_int, x_int)) invalid = true;
                const bool not_in_rdr_grid = y_int < 0 || (size_t)y_int >= rL || x_int < 0 || (size_t)x_int >= rW;
                invalid = invalid || not_in_rdr_grid;
            }
            ry[tid] = invalid ? 0.0 : y;
            rx[tid] = invalid ? 0.0 : x;
            mask[tid] = invalid;
        }
        // Geocode.cu:418-460: masked min/max and the radar block (+-5)
        double xmin = NAN, xmax = NAN, ymin = NAN, ymax = NAN;
        for (size_t k = 0; k < n; ++k) {
            if (mask[k]) continue;
            if (std::isnan(xmin) || rx[k] < xmin) xmin = rx[k];
            if (std::isnan(xmax) || rx[k] > xmax) xmax = rx[k];
            if (std::isnan(ymin) || ry[k] < ymin) ymin = ry[k];
            if (std::isnan(ymax) || ry[k] > ymax) ymax = ry[k];
        }
        const bool all_masked = std::isnan(ymin);
        size_t rg_first = 0, rg_last = 0, az_first = 0, az_last = 0, bw = 0, bl = 0;
        if (!all_masked) {
            rg_first = std::min(rW - 1, (size_t)std::floor(xmin));
            rg_last = (size_t)std::max(0.0, std::ceil(xmax) - 1);
            az_first = std::min(rL - 1, (size_t)std::floor(ymin));
            az_last = (size_t)std::max(0.0, std::ceil(ymax) - 1);
            const size_t margin = 5;
            rg_first = margin > rg_first ? 0 : rg_first - margin;
            rg_last = std::min(rW - 1, rg_last + margin);
            az_first = margin > az_first ? 0 : az_first - margin;
            az_last = std::min(rL - 1, az_last + margin);
            bw = rg_last - rg_first + 1;
            bl = az_last - az_first + 1;
        }
        for (long k = 0; k < (long)n; ++k) {
            const size_t o = (size_t)line_start * W + k;
            if (a->out_az_index) a->out_az_index[o] = mask[k] ? NAN : ry[k];
            if (a->out_rg_index) a->out_rg_index[o] = mask[k] ? NAN : rx[k];
        }
        for (int r = 0; r < a->n_rasters; ++r) {
            const double iv = a->invalid_values[r];
            const float inv = std::isnan(iv) ? std::numeric_limits<float>::quiet_NaN() : (float)iv;
            const cf* in = reinterpret_cast<const cf*>(a->input_rasters[r]);
            cf* out = reinterpret_cast<cf*>(a->output_rasters[r]) + (size_t)line_start * W;
            // interpolate, Geocode.cu:203-287, over the radar block read at
            // (rg_first, az_first) (Geocode.cu:586-600)
#pragma omp parallel for schedule(dynamic, 1024)
            for (long k = 0; k < (long)n; ++k) {
                cf val{inv, inv};
                if (bw > 0 && !mask[k]) {
                    const double rdry = ry[k] - (double)az_first;
                    const double rdrx = rx[k] - (double)rg_first;
                    const bool oob = rdrx < 4.0 || rdry < 4.0 || rdrx >= (double)bw - 4.0 || rdry >= (double)bl - 4.0;
                    if (!oob) {
                        const int xi = (int)std::floor(rdrx), yi = (int)std::floor(rdry);
                        const double fx = rdrx - (double)xi, fy = rdry - (double)yi;
                        cf chip[81];
                        for (int i = 0; i < 9; ++i)
                            for (int j = 0; j < 9; ++j) {
                                const size_t row = az_first + (size_t)(yi + i - 4);
                                const size_t col = rg_first + (size_t)(xi + j - 4);
                                chip[i * 9 + j] = in[row * rW + col];
                            }
                        val = sinc2d_chip(chip, 9, 9, 4.0 + fx, 4.0 + fy);
                    }
                }
                out[k] = val;
            }
        }
    }
    return 0;
}

// ================================================================ components
extern "C" int orc_orbit_interpolate(const orc_orbit* o, double t, double* pos, double* vel) {
    V3 p{NaN, NaN, NaN}, v{NaN, NaN, NaN};
    int st = orbit_interp(o, t, &p, &v);
    pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
    vel[0] = v.x; vel[1] = v.y; vel[2] = v.z;
    return st;
}

extern "C" double orc_interp2d_double(int method, const double* z, int ny, int nx, double x, double y) {
    switch (method) {
        case 1: return bilinear(z, nx, x, y);
        case 2: return bicubic(z, ny, nx, x, y);
        case 3: return nearest(z, nx, x, y);
        case 4: return spline2d<double>(z, ny, nx, x, y);
        case 5: return sinc2d_double(z, ny, nx, x, y);
        default: return NaN;
    }
}

// the SLC interpolator (sinc2d_chip) on a row-major complex64 table
// (interleaved re, im); out: re, im
extern "C" void orc_sinc2d_cfloat(const float* z, int ny, int nx, double x, double y, float* out) {
    const cf r = sinc2d_chip(reinterpret_cast<const cf*>(z), ny, nx, x, y);
    out[0] = r.re;
    out[1] = r.im;
}

extern "C" float orc_spline2d_float(const float* z, int ny, int nx, double x, double y) {
    return spline2d<float>(z, ny, nx, x, y);
}

extern "C" double orc_lut2d_eval(const orc_lut2d* l, double y, double x) { return lut_eval(l, y, x); }
extern "C" int orc_lut2d_contains(const orc_lut2d* l, double y, double x) { return lut_contains(l, y, x) ? 1 : 0; }
extern "C" double orc_poly2d_eval(const orc_poly2d* p, double y, double x) { return poly_eval(p, y, x); }

extern "C" int orc_proj_forward(int epsg, const double* llh, double* xyz) {
    Proj p;
    if (!p.init(epsg)) return -1;
    V3 o{0, 0, 0};
    int st = p.forward({llh[0], llh[1], llh[2]}, o);
    xyz[0] = o.x; xyz[1] = o.y; xyz[2] = o.z;
    return st;
}

extern "C" int orc_proj_inverse(int epsg, const double* xyz, double* llh) {
    Proj p;
    if (!p.init(epsg)) return -1;
    V3 o{0, 0, 0};
    int st = p.inverse({xyz[0], xyz[1], xyz[2]}, o);
    llh[0] = o.x; llh[1] = o.y; llh[2] = o.z;
    return st;
}

extern "C" void orc_lonlat_to_xyz(double a, double e2, const double* llh, double* xyz) {
    V3 o = lonlat_to_xyz(a, e2, {llh[0], llh[1], llh[2]});
    xyz[0] = o.x; xyz[1] = o.y; xyz[2] = o.z;
}

extern "C" int orc_geo2rdr(const double* llh, double a, double e2, const orc_orbit* orbit,
                           const orc_lut2d* doppler, double* aztime, double* srange,
                           double wavelength, int look_side, double threshold, int maxiter,
                           double delta_range) {
    double t0 = *aztime;
    int st = geo2rdr_detail(aztime, srange, {llh[0], llh[1], llh[2]}, a, e2, orbit, doppler,
                            wavelength, look_side, t0, threshold, maxiter, delta_range);
    return st == G_OK ? 1 : 0;
}

extern "C" void orc_sinc_table(float* out) {
    const SincTable& T = sinc_table();
    for (size_t i = 0; i < T.k.size(); ++i) out[i] = (float)T.k[i];
}

extern "C" int orc_dem_subset(const orc_dem_raster* dem, const orc_geo_grid* g, int margin,
                              int64_t* x_off, int64_t* y_off, int64_t* width, int64_t* length,
                              double* x_start, double* y_start) {
    DEM d;
    if (dem_raster_to_interp(d, dem, g, 0, g->length, g->width, margin)) return 1;
    if (!d.have_raster) { *width = 0; *length = 0; return 0; }
    *x_off = (int64_t)std::llround((d.xstart - dem->gt[0]) / dem->gt[1] - 0.5);
    *y_off = (int64_t)std::llround((d.ystart - dem->gt[3]) / dem->gt[5] - 0.5);
    *width = d.width; *length = d.length;
    *x_start = d.xstart; *y_start = d.ystart;
    return 0;
}

// ---------------------------------------------------------------- block planning
// geometry/boundingbox.cpp:434-641 (getRadarBoundingBox with min/max heights):
// the four geogrid corners at the two heights, each corner pushed outwards by
// one geogrid pixel per retry until geo2rdr converges; floor/ceil of the
// radar coordinates, the overlap checks, then the margin, clamped.
extern "C" int orc_radar_bbox(const orc_geo_grid* g, const orc_radar_grid* rg, const orc_orbit* orbit,
                              const orc_lut2d* doppler, float min_height, float max_height, int margin,
                              double threshold, int maxiter, double delta_range, int expansion_threshold,
                              int32_t* out) {
    if (max_height < min_height) return fail("max_height <  min_height");
    if (margin < 0) return fail("Margin should be a nonnegative number.");
    Proj proj;
    if (!proj.init(g->epsg)) return fail("unsupported EPSG");
    const float height_range[2] = {min_height, max_height};
    int first_az = (int)(rg->length - 1), last_az = 0;
    int first_rg = (int)(rg->width - 1), last_rg = 0;
    const int ex[2][2] = {{-1, 1}, {-1, 1}}, ey[2][2] = {{-1, -1}, {1, 1}};
    int bad = 0;
    for (size_t line = 0; line < 2; ++line) {
        const double y0 = g->start_y + g->spacing_y * line * g->length;
        for (size_t pixel = 0; pixel < 2; ++pixel) {
            const double x0 = g->start_x + g->spacing_x * pixel * g->width;
            bool corner_converge = false;
            for (int ih = 0; ih < 2; ++ih) {
                const float height = height_range[ih];
                double aztime = rg_sensing_mid(*rg);
                double srange = rg->starting_range;
                int iters = 0, geostat = 0;
                while (geostat == 0 && iters < expansion_threshold) {
                    const double x = x0 + iters * ex[line][pixel] * g->spacing_x;
                    const double y = y0 + iters * ey[line][pixel] * g->spacing_y;
                    V3 llh{0, 0, 0};
                    if (proj.inverse({x, y, 0.0}, llh) != 0) {
                        out[4] = 3; out[5] = 0;
                        return 0;   // RuntimeError: Inverse projection transformation failed
                    }
                    llh.z = height;
                    const double t0 = aztime;
                    geostat = geo2rdr_detail(&aztime, &srange, llh, WGS84_A, WGS84_E2, orbit, doppler,
                                             rg->wavelength, rg->look_side, t0, threshold, maxiter,
                                             delta_range) == G_OK;
                    iters += 1;
                }
                if (geostat == 0) continue;
                corner_converge = true;
                const double az = (aztime - rg->sensing_start) * rg->prf;
                const double r = (srange - rg->starting_range) / rg->range_pixel_spacing;
                first_az = std::min(first_az, (int)std::floor(az));
                last_az = std::max(last_az, (int)std::ceil(az));
                first_rg = std::min(first_rg, (int)std::floor(r));
                last_rg = std::max(last_rg, (int)std::ceil(r));
            }
            if (!corner_converge) bad |= 1 << (2 * line + pixel);
        }
    }
    out[0] = first_az; out[1] = last_az; out[2] = first_rg; out[3] = last_rg;
    if (bad) { out[4] = 1; out[5] = bad; return 0; }
    const int max_az = (int)(rg->length - 1), max_rg = (int)(rg->width - 1);
    int why = 0;
    if (first_az <= 0 && last_az <= 0) why |= 1;
    if (first_az >= max_az && last_az >= max_az) why |= 2;
    if (first_rg <= 0 && last_rg <= 0) why |= 4;
    if (first_rg >= max_rg && last_rg >= max_rg) why |= 8;
    if (why) { out[4] = 2; out[5] = why; return 0; }
    out[0] = std::max(first_az - margin, 0);
    out[2] = std::max(first_rg - margin, 0);
    out[1] = std::min(last_az + margin, max_az);
    out[3] = std::min(last_rg + margin, max_rg);
    out[4] = 0; out[5] = 0;
    return 0;
}

// geometry/DEMInterpolator.cpp:515-560 (computeMinMaxMeanHeight): NaN samples
// are skipped and leave the mean's denominator.
extern "C" void orc_dem_stats(const float* z, int64_t length, int64_t width, float* mn, float* mx, double* mean,
                              int64_t* n_valid) {
    float lo = std::numeric_limits<float>::max(), hi = -std::numeric_limits<float>::max();
    double sum = 0.0;
    int64_t n = length * width;
    for (int64_t i = 0; i < length * width; ++i) {
        const float v = z[i];
        if (std::isnan(v)) { --n; continue; }
        hi = std::max(v, hi);
        lo = std::min(v, lo);
        sum += v;
    }
    *mn = lo; *mx = hi; *mean = sum / n; *n_valid = n;
}

// ---------------------------------------------------------------- metadata cubes
namespace {
// core/Ellipsoid.h:197-231 (Vermeille 2002)
V3 xyz_to_lonlat(double a, double e2, V3 x) {
    const double e4 = e2 * e2, a2 = a * a;
    const double p = (std::pow(x.x, 2) + std::pow(x.y, 2)) / a2;
    const double q = ((1. - e2) * std::pow(x.z, 2)) / a2;
    const double r = (p + q - e4) / 6.;
    const double s = (e4 * p * q) / (4. * std::pow(r, 3));
    const double t = std::pow(1. + s + std::sqrt(s * (2. + s)), (1. / 3.));
    const double u = r * (1. + t + (1. / t));
    const double rv = std::sqrt(std::pow(u, 2) + (e4 * q));
    const double w = (e2 * (u + rv - q)) / (2. * rv);
    const double k = std::sqrt(u + rv + std::pow(w, 2)) - w;
    const double d = (k * std::sqrt(std::pow(x.x, 2) + std::pow(x.y, 2))) / (k + e2);
    V3 llh;
    llh.y = std::atan2(x.z, d);
    llh.x = std::atan2(x.y, x.x);
    llh.z = ((k + e2 - 1.) * std::sqrt(std::pow(d, 2) + std::pow(x.z, 2))) / k;
    return llh;
}

// core/DenseMatrix.h:73-79 (xyzToEnu) applied to v
V3 xyz_to_enu(double lat, double lon, V3 v) {
    return {-std::sin(lon) * v.x + std::cos(lon) * v.y + 0. * v.z,
            -std::sin(lat) * std::cos(lon) * v.x + -std::sin(lat) * std::sin(lon) * v.y + std::cos(lat) * v.z,
            std::cos(lat) * std::cos(lon) * v.x + std::cos(lat) * std::sin(lon) * v.y + std::sin(lat) * v.z};
}

V3 normalized(V3 v) {
    const double n = norm(v);
    return {v.x / n, v.y / n, v.z / n};
}
}  // namespace

// geometry/metadataCubes.cpp:276-489 (makeRadarGridCubes) with
// writeVectorDerivedCubes (:74-274) for the outputs isce3 writes in the GSLC
// workflow: per height layer, every geogrid point solves geo2rdr with the
// grid Doppler from the previous point's result (sensingMid at the start and
// after a failure), then with the native Doppler for the platform position.
// Outputs are n_heights x length x width, NaN where not solved; NULL skips one.
extern "C" int orc_radar_grid_cubes(const orc_radar_grid* rg, const orc_geo_grid* g, const double* heights,
                                    int n_heights, const orc_orbit* orbit, const orc_lut2d* native_doppler,
                                    const orc_lut2d* grid_doppler, double threshold, int maxiter,
                                    double delta_range, double* slant_range, double* azimuth_time,
                                    float* incidence, float* los_x, float* los_y, float* along_x,
                                    float* along_y, float* elevation, double* ground_velocity, int nthreads) {
    Proj proj;
    if (!proj.init(g->epsg)) return fail("unsupported EPSG");
    const int64_t L = g->length, W = g->width, plane = L * W;
    const double fnan = std::numeric_limits<float>::quiet_NaN();
    auto fill = [&](auto* p, double v) {
        if (p) for (int64_t i = 0; i < plane * n_heights; ++i) p[i] = (std::remove_reference_t<decltype(*p)>)v;
    };
    fill(slant_range, NaN); fill(azimuth_time, NaN); fill(incidence, fnan); fill(los_x, fnan); fill(los_y, fnan);
    fill(along_x, fnan); fill(along_y, fnan); fill(elevation, fnan); fill(ground_velocity, NaN);
    const bool vec = incidence || los_x || los_y || along_x || along_y || elevation || ground_velocity;
    const double mid_range = 0.5 * (rg->starting_range + rg_ending_range(*rg));
    int proj_fail = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : proj_fail)
    for (int hc = 0; hc < n_heights; ++hc) {
        double az_t = rg_sensing_mid(*rg), nat_t = rg_sensing_mid(*rg);
        double sr = mid_range, nat_sr = mid_range;
        const double height = heights[hc];
        for (int64_t i = 0; i < L; ++i) {
            const double pos_y = g->start_y + (0.5 + i) * g->spacing_y;
            for (int64_t j = 0; j < W; ++j) {
                const double pos_x = g->start_x + (0.5 + j) * g->spacing_x;
                V3 llh{0, 0, 0};
                if (proj.inverse({pos_x, pos_y, height}, llh) != 0) { proj_fail = 1; continue; }
                const int64_t k = hc * plane + i * W + j;
                double t0 = az_t;
                if (geo2rdr_detail(&az_t, &sr, llh, WGS84_A, WGS84_E2, orbit, grid_doppler, rg->wavelength,
                                   rg->look_side, t0, threshold, maxiter, delta_range) != G_OK) {
                    az_t = rg_sensing_mid(*rg);
                    sr = mid_range;
                    continue;
                }
                if (slant_range) slant_range[k] = sr;
                if (azimuth_time) azimuth_time[k] = az_t;
                if (!vec) continue;
                t0 = nat_t;
                if (geo2rdr_detail(&nat_t, &nat_sr, llh, WGS84_A, WGS84_E2, orbit, native_doppler, rg->wavelength,
                                   rg->look_side, t0, threshold, maxiter, delta_range) != G_OK) {
                    nat_t = rg_sensing_mid(*rg);
                    nat_sr = mid_range;
                    continue;
                }
                V3 sat, vel;
                if (orbit_interp(orbit, nat_t, &sat, &vel) != 0) continue;
                const V3 target = lonlat_to_xyz(WGS84_A, WGS84_E2, llh);
                if (ground_velocity) {
                    const double slant = norm(sub(target, sat));
                    const double rt = norm(target), rp = norm(sat);
                    const double cos_alpha = ((rt * rt + rp * rp - slant * slant) / (2 * rt * rp));
                    ground_velocity[k] = cos_alpha * rt * norm(vel) / rp;
                }
                const V3 look = normalized(sub(sat, target));
                if (elevation) {
                    const V3 sat_llh = xyz_to_lonlat(WGS84_A, WGS84_E2, sat);
                    const V3 le = normalized(xyz_to_enu(sat_llh.y, sat_llh.x, look));
                    elevation[k] = (float)(std::acos(le.z) * 180.0 / M_PI);
                }
                const V3 le = normalized(xyz_to_enu(llh.y, llh.x, look));
                if (incidence) incidence[k] = (float)(std::acos(std::abs(le.z)) * 180.0 / M_PI);
                if (los_x) los_x[k] = (float)le.x;
                if (los_y) los_y[k] = (float)le.y;
                if (along_x || along_y) {
                    const V3 at = normalized(xyz_to_enu(llh.y, llh.x, vel));
                    if (along_x) along_x[k] = (float)at.x;
                    if (along_y) along_y[k] = (float)at.y;
                }
            }
        }
    }
    if (proj_fail) return fail("Inverse projection transformation failed");
    return 0;
}

// ---------------------------------------------------------------- raster interpolators
// The device interpolators of the CUDA raster geocoder (cuda/core/
// gpuNearestNeighborInterpolator.cu:8-15, gpuBilinearInterpolator.cu:78-108,
// gpuBicubicInterpolator.cu:104-188, gpuSpline2dInterpolator.cu _initSpline /
// _spline / interpolate with order 6, gpuSinc2dInterpolator.cu:103-140 over
// the chip of cuda/geocode/Geocode.cu:243-277), on one real component of a
// sample: the reference's complex (thrust) arithmetic meets only real
// weights, so each component follows the real arithmetic.
namespace {
template <typename S>
struct RView {
    const S* z;
    int64_t nx;
    int nc, c;
    S operator()(int64_t r, int64_t col) const { return z[(r * nx + col) * nc + c]; }
};

template <typename S>
S r_nearest(double x, double y, const RView<S>& z) {
    return z((int64_t)std::round(y), (int64_t)std::round(x));
}

template <typename S>
S r_bilinear(double x, double y, const RView<S>& z) {
    const size_t x1 = std::floor(x), x2 = std::ceil(x), y1 = std::floor(y), y2 = std::ceil(y);
    const S q11 = z(y1, x1), q12 = z(y2, x1), q21 = z(y1, x2), q22 = z(y2, x2);
    if ((y1 == y2) && (x1 == x2)) return q11;
    if (y1 == y2) return ((S)((x2 - x) / (x2 - x1)) * q11) + ((S)((x - x1) / (x2 - x1)) * q21);
    if (x1 == x2) return ((S)((y2 - y) / (y2 - y1)) * q11) + ((S)((y - y1) / (y2 - y1)) * q12);
    return ((q11 * (S)((x2 - x) * (y2 - y))) / (S)((x2 - x1) * (y2 - y1))) +
           ((q21 * (S)((x - x1) * (y2 - y))) / (S)((x2 - x1) * (y2 - y1))) +
           ((q12 * (S)((x2 - x) * (y - y1))) / (S)((x2 - x1) * (y2 - y1))) +
           ((q22 * (S)((x - x1) * (y - y1))) / (S)((x2 - x1) * (y2 - y1)));
}

const double BICUBIC_W[256] = {
    1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,     0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0,
    -3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1, 0, 0, 0, 0,  2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0,
    0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,     0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0,
    0, 0, 0, 0, -3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1,  0, 0, 0, 0, 2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1,
    -3, 3, 0, 0, -2, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,  0, 0, 0, 0, 0, 0, 0, 0, -3, 3, 0, 0, -2, -1, 0, 0,
    9, -9, 9, -9, 6, 3, -3, -6, 6, -6, -3, 3, 4, 2, 1, 2,
    -6, 6, -6, 6, -4, -2, 2, 4, -3, 3, 3, -3, -2, -1, -1, -2,
    2, -2, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,    0, 0, 0, 0, 0, 0, 0, 0, 2, -2, 0, 0, 1, 1, 0, 0,
    -6, 6, -6, 6, -3, -3, 3, 3, -4, 4, 2, -2, -2, -2, -1, -1,
    4, -4, 4, -4, 2, 2, -2, -2, 2, -2, -2, 2, 1, 1, 1, 1};

template <typename S>
S r_bicubic(double x, double y, const RView<S>& z) {
    const int64_t x1 = std::floor(x), x2 = std::ceil(x), y1 = std::floor(y), y2 = std::ceil(y);
    const S denom = S(2.0), scale = S(0.25);
    const S zz[4] = {z(y1, x1), z(y1, x2), z(y2, x2), z(y2, x1)};
    const S dzdx[4] = {(z(y1, x1 + 1) - z(y1, x1 - 1)) / denom, (z(y1, x2 + 1) - z(y1, x2 - 1)) / denom,
                       (z(y2, x2 + 1) - z(y2, x2 - 1)) / denom, (z(y2, x1 + 1) - z(y2, x1 - 1)) / denom};
    // the reference's y-derivative stencils, as written there
    const S dzdy[4] = {(z(y1 + 1, x1) - z(y1 - 1, x1)) / denom, (z(y1 + 1, x2 + 1) - z(y1 - 1, x2)) / denom,
                       (z(y2 + 1, x2 + 1) - z(y2 - 1, x2)) / denom, (z(y2 + 1, x1 + 1) - z(y2 - 1, x1)) / denom};
    const int64_t xs[4] = {x1, x2, x2, x1}, ys[4] = {y1, y1, y2, y2};
    S dzdxy[4];
    for (int k = 0; k < 4; ++k)
        dzdxy[k] = scale * (z(ys[k] + 1, xs[k] + 1) - z(ys[k] - 1, xs[k] + 1) - z(ys[k] + 1, xs[k] - 1) +
                            z(ys[k] - 1, xs[k] - 1));
    S q[16];
    for (int i = 0; i < 4; ++i) {
        q[i] = zz[i];
        q[i + 4] = dzdx[i];
        q[i + 8] = dzdy[i];
        q[i + 12] = dzdxy[i];
    }
    S c[16];
    for (int i = 0; i < 16; ++i) {
        S qq(0.0);
        for (int j = 0; j < 16; ++j) qq += (S)(BICUBIC_W[i * 16 + j]) * q[j];
        c[i] = qq;
    }
    const S t = x - x1, u = y - y1;
    S ret = 0.0;
    for (int i = 3; i >= 0; i--) ret = t * ret + ((c[i * 4 + 3] * u + c[i * 4 + 2]) * u + c[i * 4 + 1]) * u + c[i * 4];
    return ret;
}

template <typename S>
void r_init_spline(const S* Y, int n, S* R, S* Q) {
    Q[0] = 0.0;
    R[0] = 0.0;
    for (int i = 1; i < n - 1; ++i) {
        const auto p = 1.0 / (0.5 * Q[i - 1] + 2.0);
        Q[i] = -0.5 * p;
        R[i] = (3 * (Y[i + 1] - 2 * Y[i] + Y[i - 1]) - 0.5 * R[i - 1]) * p;
    }
    R[n - 1] = 0.0;
    for (int i = (n - 2); i > 0; --i) R[i] = Q[i] * R[i + 1] + R[i];
}

template <typename S>
S r_spline(double x, const S* Y, int n, const S* R) {
    if (x < 1.0) return Y[0] + (x - 1.0) * (Y[1] - Y[0] - (R[1] / 6.0));
    if (x > n) return Y[n - 1] + ((x - n) * (Y[n - 1] - Y[n - 2] + (R[n - 2] / 6.)));
    const int j = int(std::floor(x));
    const auto xx = x - j;
    const auto t0 = Y[j] - Y[j - 1] - (R[j - 1] / 3.0) - (R[j] / 6.0);
    const auto t1 = xx * ((R[j - 1] / 2.0) + (xx * ((R[j] - R[j - 1]) / 6)));
    return Y[j - 1] + (xx * (t0 + t1));
}

template <typename S>
S r_biquintic(double x, double y, const RView<S>& z, int64_t ny) {
    const int order = 6;
    int i0 = y, j0 = x;                  // order even: truncation
    i0 = i0 - (order / 2) + 1;
    j0 = j0 - (order / 2) + 1;
    S A[order], R[order], Q[order], HC[order];
    for (int i = 0; i < order; ++i) {
        const int64_t indi = std::min(std::max((int64_t)(i0 + i), (int64_t)0), ny - 2);
        for (int j = 0; j < order; ++j) {
            const int64_t indj = std::min(std::max((int64_t)(j0 + j), (int64_t)0), z.nx - 2);
            A[j] = z(indi + 1, indj + 1);
        }
        r_init_spline(A, order, R, Q);
        HC[i] = r_spline(x - j0, A, order, R);
    }
    r_init_spline(HC, order, R, Q);
    return (S)(r_spline(y - i0, HC, order, R));
}

template <typename S>
S r_sinc(double x, double y, const RView<S>& z, const std::vector<double>& table) {
    const int xi = (int)std::floor(x), yi = (int)std::floor(y);
    const double X = SINC_HALF + (x - xi), Y = SINC_HALF + (y - yi);
    const int ix = (int)std::floor(X), iy = (int)std::floor(Y);
    if (!((ix >= SINC_HALF - 1) && (ix <= SINC_ONE - SINC_HALF - 1) && (iy >= SINC_HALF - 1) &&
          (iy <= SINC_ONE - SINC_HALF - 1)))
        return S(0.0);
    const double frpx = X - ix, frpy = Y - iy;
    const int intpx = ix + SINC_HALF, intpy = iy + SINC_HALF;
    const int ifracx = std::min(std::max(0, int(frpx * SINC_SUB)), SINC_SUB - 1);
    const int ifracy = std::min(std::max(0, int(frpy * SINC_SUB)), SINC_SUB - 1);
    S v(0.0);
    for (int i = 0; i < SINC_LEN; i++)
        for (int j = 0; j < SINC_LEN; j++)
            v += z(yi + (intpy - i) - SINC_HALF, xi + (intpx - j) - SINC_HALF) *
                 S(table[ifracy * SINC_LEN + i]) * S(table[ifracx * SINC_LEN + j]);
    return v;
}

template <typename S>
void r_interpolate(const S* raster, const double* az, const double* rg, int64_t n, int64_t L, int64_t W, S* out,
                   int nc, int method, double invalid) {
    std::vector<double> table;
    if (method == 0) {
        const SincTable& T = sinc_table();
        table.assign(T.k.begin(), T.k.end());
    }
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const double y = az[k], x = rg[k];
        const bool ok = !(std::isnan(x) || std::isnan(y) || x < 4.0 || y < 4.0 || x >= W - 4.0 || y >= L - 4.0);
        for (int c = 0; c < nc; ++c) {
            S v = (S)invalid;
            if (ok) {
                const RView<S> z{raster, W, nc, c};
                switch (method) {
                case 0: v = r_sinc(x, y, z, table); break;
                case 1: v = r_bilinear(x, y, z); break;
                case 2: v = r_bicubic(x, y, z); break;
                case 3: v = r_nearest(x, y, z); break;
                default: v = r_biquintic(x, y, z, L); break;
                }
            }
            out[k * nc + c] = v;
        }
    }
}
}  // namespace

// cuda/geocode/Geocode.cu:203-287: raster samples at per-pixel radar
// coordinates (NaN: masked).  gdal_type: 1 Byte, 2 UInt16, 4 UInt32,
// 6 Float32, 7 Float64, 10 CFloat32, 11 CFloat64.
extern "C" int orc_interpolate_raster(const double* az, const double* rg, int64_t n, const void* raster, int64_t L,
                                      int64_t W, void* out, int gdal_type, int method, double invalid) {
    auto uint_nearest = [&](auto* src, auto* dst) {
        using U = std::remove_pointer_t<decltype(dst)>;
        for (int64_t k = 0; k < n; ++k) {
            const double y = az[k], x = rg[k];
            const bool ok = !(std::isnan(x) || std::isnan(y) || x < 4.0 || y < 4.0 || x >= W - 4.0 || y >= L - 4.0);
            dst[k] = ok ? src[(int64_t)std::round(y) * W + (int64_t)std::round(x)] : (U)invalid;
        }
    };
    switch (gdal_type) {
    case 6: r_interpolate((const float*)raster, az, rg, n, L, W, (float*)out, 1, method, invalid); break;
    case 10: r_interpolate((const float*)raster, az, rg, n, L, W, (float*)out, 2, method, invalid); break;
    case 7: r_interpolate((const double*)raster, az, rg, n, L, W, (double*)out, 1, method, invalid); break;
    case 11: r_interpolate((const double*)raster, az, rg, n, L, W, (double*)out, 2, method, invalid); break;
    case 1: uint_nearest((const uint8_t*)raster, (uint8_t*)out); break;
    case 2: uint_nearest((const uint16_t*)raster, (uint16_t*)out); break;
    case 4: uint_nearest((const uint32_t*)raster, (uint32_t*)out); break;
    default: return fail("unsupported raster data type");
    }
    return 0;
}
