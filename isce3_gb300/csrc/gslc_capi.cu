// C ABI of libgslc.so: contexts, argument checks, host-side precomputation
// (sinc table, orbit polynomials, DEM window) and kernel launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/gslc.h"
#include "gslc_kernels.cuh"

using namespace gslc;

// row bands of gslc_geocode_slc_to_host (copies of a band overlap the next bands' kernels)
constexpr int GSLC_HOST_BANDS = 4;

struct gslc_ctx {
    int device = 0;
    float* d_sinc = nullptr;        // SINC_SUB * SINC_LEN
    int32_t* d_err = nullptr;
    int32_t* h_err = nullptr;       // pinned
    double* d_orbit = nullptr;
    size_t orbit_cap = 0;           // doubles
    int64_t launches = 0;
    int timing = 0;                 // record CUDA events around the kernels
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float ms_geocode = 0.f, ms_deramp = 0.f;
    int cube_passes = 0;            // passes of the last gslc_make_radar_grid_cubes
    double* d_sinc64 = nullptr;     // the sinc table in double (raster interpolation), on first use
    cudaStream_t copy_stream = nullptr;   // device-to-host copies of gslc_geocode_slc_to_host, on first use
    cudaEvent_t band_ev[GSLC_HOST_BANDS + 1] = {};
    int64_t stage_wait = 0;         // SM clocks of the orbit-table wait; 0: STAGE_WAIT_DEFAULT
    // gslc_geocode_slc_host_io: upload stream, second compute stream, events, re-runs of the last call
    cudaStream_t h2d_stream = nullptr, aux_stream = nullptr;
    std::vector<cudaEvent_t> io_ev;
    int io_reruns = 0;
    bool no_alloc = false;          // the allocation-free entry point's stand-in context
    // the host tables (build_orbit_table) of the last few orbits, keyed by
    // the descriptor and the state vectors, most recent first: calls that
    // reuse an orbit skip rebuilding them
    struct OrbitTables {
        std::vector<double> key, coef;
        Orbit ob{};
    };
    std::vector<OrbitTables> orbit_cache;
    std::string err;
};

namespace {

int set_err(gslc_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}

int cuda_err(gslc_ctx* c, cudaError_t e, const char* where) {
    return set_err(c, GSLC_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// The kernels' device error word: bit 0 a projection inverse failed; bit 1
// a wait for the orbit tables' copy into shared memory ran out (the global
// tables were read instead, so the outputs are complete and correct); bit 2
// a block's final wait for its copy ran out too.
int device_status(gslc_ctx* c, int32_t word) {
    if (word & 1) return set_err(c, GSLC_EPROJ, "Inverse projection transformation failed");
    if (word & 4) return set_err(c, GSLC_ETIMEOUT, "an orbit table copy into shared memory did not complete");
    if (word & 2) return set_err(c, GSLC_ETIMEOUT, "the wait for the orbit table copy into shared memory ran out");
    return GSLC_OK;
}

// core/Sinc2dInterpolator.cpp:12-40 and :98-115 — Hann-weighted sinc,
// SINC_LEN taps x SINC_SUB phases, each phase normalised to unit sum, then
// cast to float at use (Sinc2dInterpolator.cpp:88-90).
std::vector<double> make_sinc_table_double() {
    const int filtercoef = SINC_SUB * SINC_LEN;
    std::vector<double> filter(filtercoef, 0.0);
    const double beta = 1.0, pedestal = 0.0;
    const double wgthgt = (1.0 - pedestal) / 2.0;
    const double soff = (filtercoef - 1.) / 2.;
    for (int i = 0; i < filtercoef; i++) {
        const double wgt = (1. - wgthgt) + (wgthgt * std::cos((M_PI * (i - soff)) / soff));
        const double s = (std::floor(i - soff) * beta) / (1. * SINC_SUB);
        const double fct = ((s != 0.) ? (std::sin(M_PI * s) / (M_PI * s)) : 1.);
        filter[i] = fct * wgt;
    }
    std::vector<double> table((size_t)filtercoef);
    for (int i = 0; i < SINC_SUB; ++i) {
        double ssum = 0.0;
        for (int j = 0; j < SINC_LEN; ++j) ssum += filter[i + SINC_SUB * j];
        for (int j = 0; j < SINC_LEN; ++j) {
            filter[i + SINC_SUB * j] /= ssum;
            table[(size_t)i * SINC_LEN + j] = filter[i + SINC_SUB * j];
        }
    }
    return table;
}

std::vector<float> make_sinc_table() {
    const std::vector<double> d = make_sinc_table_double();
    std::vector<float> table(d.size());
    for (size_t i = 0; i < d.size(); ++i) table[i] = (float)d[i];
    return table;
}

// Data-independent part of _initSpline for n = 6
// (core/Spline2dInterpolator.cpp:95-100), in FP32 like the reference.
SplineConst make_spline_const() {
    SplineConst k{};
    float q_prev = 0.0f;
    for (int i = 1; i < 5; ++i) {
        volatile float half_q = 0.5f * q_prev;   // keep mul and add separately rounded
        const float p = 1.0f / (half_q + 2.0f);
        k.p[i] = p;
        k.q[i] = -0.5f * p;
        q_prev = k.q[i];
    }
    k.p[0] = k.q[0] = 0.0f;
    // the CUDA interpolator's recurrence: p = 1.0 / (0.5 * Q + 2.0) in FP64,
    // Q = -0.5 * p stored to FP32 (cuda/core/gpuSpline2dInterpolator.cu:89-92)
    float qd_prev = 0.0f;
    for (int i = 1; i < 5; ++i) {
        volatile double half_q = 0.5 * (double)qd_prev;
        const double p = 1.0 / (half_q + 2.0);
        k.pd[i] = p;
        k.qd[i] = (float)(-0.5 * p);
        qd_prev = k.qd[i];
    }
    k.pd[0] = 0.0;
    k.qd[0] = 0.0f;
    return k;
}

// ---- double-double helpers (Knuth TwoSum, FMA-based TwoProd) --------------
struct dd { double hi, lo; };
dd two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return two_sum(s.hi, s.lo);
}
dd dd_mul_d(dd a, double b) {
    const double p = a.hi * b;
    const double e = std::fma(a.hi, b, -p);
    return two_sum(p, e + a.lo * b);
}
dd dd_div_d(dd a, double b) {
    const double q1 = a.hi / b;
    dd r = dd_add(a, dd_mul_d({q1, 0.0}, -b));
    const double q2 = r.hi / b;
    return two_sum(q1, q2);
}

// Integer-coefficient polynomials (exact in double for these sizes).
using P8 = std::vector<double>;
P8 pmul(const P8& a, const P8& b) {
    P8 r(a.size() + b.size() - 1, 0.0);
    for (size_t i = 0; i < a.size(); ++i)
        for (size_t j = 0; j < b.size(); ++j) r[i + j] += a[i] * b[j];
    return r;
}
// q(u + c): Taylor shift, exact for dyadic c and these magnitudes
P8 pshift(const P8& q, double c) {
    P8 r(q.size(), 0.0);
    for (size_t k = 0; k < q.size(); ++k) {
        // (u + c)^k = sum_m C(k,m) c^(k-m) u^m
        double binom = 1.0;
        for (size_t m = 0; m <= k; ++m) {
            if (m > 0) binom = binom * (double)(k - m + 1) / (double)m;
            r[m] += q[k] * binom * std::pow(c, (double)(k - m));
        }
    }
    return r;
}

// Expansion of the 4-point Hermite interpolant
// (core/detail/InterpolateOrbit.icc:10-109) on each state-vector interval.
// With s = (t - t_idx)/spacing and nodes s = 0..3:
//   pos(s) = sum_i L_i(s)^2 [(1 - 2 sigma_i (s - i)) P_i + spacing (s - i) V_i]
// where L_i is the Lagrange basis and sigma_i = sum_{j != i} 1/(i - j).
// Stored around u = s - 1.5 and P_ref = P_{idx+1}.
void make_orbit_coeffs(const gslc_orbit& o, std::vector<double>& out) {
    const int npieces = o.n - 3;
    out.assign((size_t)npieces * ORB_STRIDE, 0.0);
    const P8 s1{0.0, 1.0};
    auto lin = [](double a, double b) { return P8{a, b}; };  // a + b s
    P8 N[4] = {pmul(pmul(lin(-1, 1), lin(-2, 1)), lin(-3, 1)), pmul(pmul(s1, lin(-2, 1)), lin(-3, 1)),
               pmul(pmul(s1, lin(-1, 1)), lin(-3, 1)), pmul(pmul(s1, lin(-1, 1)), lin(-2, 1))};
    const P8 Lp[4] = {lin(3, 11), lin(0, 27), lin(81, -27), lin(36, -11)};  // 108 * L_i^2 factor * f0_i / N_i^2
    const double cB[4] = {1, 9, 9, 1};                                      // 36 / D_i^2
    P8 A[4], B[4];
    for (int i = 0; i < 4; ++i) {
        const P8 n2 = pmul(N[i], N[i]);
        A[i] = pshift(pmul(n2, Lp[i]), 1.5);                   // = 108 * A_i(u)
        P8 bi = pmul(n2, lin(-(double)i, 1));
        for (double& v : bi) v *= cB[i];
        B[i] = pshift(bi, 1.5);                                // = 36 * B_i(u)
    }
    for (int idx = 0; idx < npieces; ++idx) {
        double* c = out.data() + (size_t)idx * ORB_STRIDE;
        for (int d = 0; d < 3; ++d) {
            const double pref = o.pos[(idx + 1) * 3 + d];
            c[d] = pref;
            double a[8];
            for (int k = 0; k < 8; ++k) {
                dd sa{0.0, 0.0}, sb{0.0, 0.0};
                for (int i = 0; i < 4; ++i) {
                    const double dp = o.pos[(idx + i) * 3 + d] - pref;
                    sa = dd_add(sa, dd_mul_d({dp, 0.0}, A[i][k]));
                    sb = dd_add(sb, dd_mul_d({o.vel[(idx + i) * 3 + d], 0.0}, B[i][k]));
                }
                dd term = dd_add(dd_div_d(sa, 108.0), dd_mul_d(dd_div_d(sb, 36.0), o.spacing));
                a[k] = term.hi + term.lo;
                c[3 + d * 8 + k] = a[k];
            }
            for (int k = 0; k < 7; ++k) c[27 + d * 7 + k] = (double)(k + 1) * a[k + 1] / o.spacing;
        }
    }
}

dd dd_mul(dd a, dd b) {
    const double p = a.hi * b.hi;
    const double e = std::fma(a.hi, b.hi, -p);
    return two_sum(p, e + (a.hi * b.lo + a.lo * b.hi));
}
dd dd_recip(dd a) {
    const double q1 = 1.0 / a.hi;
    const dd r = dd_add({1.0, 0.0}, dd_mul(a, {-q1, 0.0}));
    return two_sum(q1, r.hi / a.hi);
}
double dd_round(dd a) { return a.hi + a.lo; }

// r(w) = q(w + c) for an integer c in {-1, 0, 1}, in double-double
void shift_poly_dd(const double* q, int n, int c, dd* r) {
    double binom[8][8] = {};
    for (int k = 0; k < 8; ++k) {
        binom[k][0] = binom[k][k] = 1.0;
        for (int m = 1; m < k; ++m) binom[k][m] = binom[k - 1][m - 1] + binom[k - 1][m];
    }
    for (int m = 0; m < n; ++m) r[m] = {0.0, 0.0};
    for (int k = 0; k < n; ++k)
        for (int m = 0; m <= k; ++m) {
            double cp = 1.0;                        // c^(k - m), with 0^0 = 1
            for (int i = 0; i < k - m; ++i) cp *= c;
            if (cp != 0.0) r[m] = dd_add(r[m], dd_mul_d({q[k], 0.0}, binom[k][m] * cp));
        }
}

// Newton tables of every segment (SEG_STRIDE layout, gslc_math.cuh) from the
// piece coefficients of make_orbit_coeffs.  H = a . b and W = |b|^2 are
// formed in double-double from the rounded a, b the kernel evaluates;
// G = 1/W is W's reciprocal power series.  Returns the highest H and G
// degree needed over the segments, and div = 1 where G would need more
// than 12 terms (the kernel then divides).
void make_orbit_segments(const gslc_orbit& o, const double* piece, double* out, int& nh_max, int& ng_max, int& div,
                         int& a7, double& b6s, double& h6s) {
    const int nseg = o.n - 1;
    nh_max = 0;
    ng_max = 0;
    div = 0;
    a7 = 0;
    b6s = 0.0;
    h6s = 0.0;
    for (int j = 0; j < nseg; ++j) {
        const int idx = std::min(std::max(j - 1, 0), o.n - 4);
        const int c = j - idx - 1;                 // u = w + c
        const double* pc = piece + (size_t)idx * ORB_STRIDE;
        double* s = out + (size_t)j * SEG_STRIDE;
        std::fill(s, s + SEG_STRIDE, 0.0);
        for (int d = 0; d < 3; ++d) s[d] = pc[d];
        s[SEG_T] = std::fma((double)j, o.spacing, o.t0);
        double a[3][8], b[3][7];
        for (int d = 0; d < 3; ++d) {
            dd ta[8], tb[7];
            shift_poly_dd(pc + 3 + d * 8, 8, c, ta);
            shift_poly_dd(pc + 27 + d * 7, 7, c, tb);
            for (int k = 0; k < 8; ++k) s[SEG_A + d * 8 + k] = a[d][k] = dd_round(ta[k]);
            for (int k = 0; k < 7; ++k) s[SEG_B + d * 7 + k] = b[d][k] = dd_round(tb[k]);
        }
        dd H[SEG_NH], W[SEG_NG], G[SEG_NG];
        for (int k = 0; k < SEG_NH; ++k) H[k] = {0.0, 0.0};
        for (int k = 0; k < SEG_NG; ++k) W[k] = {0.0, 0.0};
        for (int d = 0; d < 3; ++d)
            for (int i = 0; i < 7; ++i) {
                for (int k = 0; k < 8; ++k) H[i + k] = dd_add(H[i + k], dd_mul({a[d][k], 0.0}, {b[d][i], 0.0}));
                for (int k = 0; k < 7; ++k) W[i + k] = dd_add(W[i + k], dd_mul({b[d][k], 0.0}, {b[d][i], 0.0}));
            }
        const dd g0 = dd_recip(W[0]);
        G[0] = g0;
        for (int k = 1; k < SEG_NG; ++k) {
            dd acc{0.0, 0.0};
            for (int m = 1; m <= k; ++m) acc = dd_add(acc, dd_mul(W[m], G[k - m]));
            G[k] = dd_mul(acc, {-g0.hi, -g0.lo});
        }
        for (int k = 0; k < SEG_NH; ++k) s[SEG_H + k] = dd_round(H[k]);
        for (int k = 0; k < SEG_NG; ++k) s[SEG_G + k] = dd_round(G[k]);
        // H degree: the tail over |w| <= 1/2 moves the Newton step by < 1e-13 s.
        // On 10 s state vectors the terms above degree 5 are the rounding
        // noise of the product (~1e-15 s), and the residual's own rounding
        // (|D.b_0| ~ 1e10 m^2/s at 2^-53) is ~1e-14 s; the reference's
        // azimuth times carry ~1e-11 s of orbit-interpolation rounding.
        int nh = SEG_NH - 1;
        {
            double tail = 0.0;
            const double lim = 1e-13 * std::fabs(W[0].hi);
            while (nh > 0) {
                const double t = tail + std::fabs(s[SEG_H + nh]) * std::ldexp(1.0, -nh);
                if (t > lim) break;
                tail = t;
                --nh;
            }
        }
        // G degree: the lowest whose truncated, rounded series times W is
        // within 2^-40 of 1 on 65 points of the segment.  G only scales the
        // step (the iteration's fixed point is fn = 0 whatever G is): a
        // relative error e in G changes each step by e of itself, which the
        // next residual corrects (10 s state vectors: degree 3)
        int ng = -1;
        for (int K = 1; K < SEG_NG && ng < 0; ++K) {
            double worst = 0.0;
            for (int q = 0; q <= 64; ++q) {
                const double w = -0.5 + q / 64.0;
                dd gv{s[SEG_G + K], 0.0}, wv = W[SEG_NG - 1];
                for (int k = K - 1; k >= 0; --k) gv = dd_add(dd_mul_d(gv, w), {s[SEG_G + k], 0.0});
                for (int k = SEG_NG - 2; k >= 0; --k) wv = dd_add(dd_mul_d(wv, w), W[k]);
                const dd e = dd_add(dd_mul(gv, wv), {-1.0, 0.0});
                worst = std::max(worst, std::fabs(e.hi));
            }
            if (worst <= std::ldexp(1.0, -40)) ng = K;
        }
        if (ng < 0) {
            div = 1;
            ng = SEG_NG - 1;
        }
        // position degree 7: kept while its term over |w| <= 1/2 reaches
        // 1e-11 m (slant ranges of ~1e6 m round at ~1e-10 m)
        for (int d = 0; d < 3; ++d)
            if (std::fabs(s[SEG_A + d * 8 + 7]) * std::ldexp(1.0, -7) >= 1e-11) a7 = 1;
        // the residual's degree-6 term D.b_6 - h_6 over |w| <= 1/2, as a step
        // (divided by |v|^2): |D| b6s + h6s seconds at most (residual_degree)
        {
            const double b6 = std::sqrt(b[0][6] * b[0][6] + b[1][6] * b[1][6] + b[2][6] * b[2][6]);
            const double scale = std::ldexp(1.0, -6) / std::fabs(W[0].hi);
            b6s = std::max(b6s, b6 * scale);
            h6s = std::max(h6s, std::fabs(s[SEG_H + 6]) * scale);
        }
        nh_max = std::max(nh_max, nh);
        ng_max = std::max(ng_max, ng);
    }
}

// The device orbit table of o (pieces, their float pairs, the Newton
// segments; orbit_table_doubles) and the Orbit descriptor, its table
// pointers left null for bind_orbit.
void build_orbit_table(const gslc_orbit& o, std::vector<double>& coef, Orbit& ob) {
    if (o.method == 1) {
        // Legendre: the state vectors themselves (positions, then
        // velocities), interpolated at each iterate as the reference does;
        // the table keeps the Hermite size so that capacities match
        coef.assign(orbit_table_doubles(o.n), 0.0);
        std::memcpy(coef.data(), o.pos, sizeof(double) * 3 * (size_t)o.n);
        std::memcpy(coef.data() + 3 * (size_t)o.n, o.vel, sizeof(double) * 3 * (size_t)o.n);
        ob = Orbit{};
        ob.t0 = o.t0;
        ob.spacing = o.spacing;
        ob.inv_spacing = 1.0 / o.spacing;
        ob.t_end = o.t0 + (o.n - 1) * o.spacing;
        ob.n = o.n;
        ob.n_pieces = o.n - 3;
        ob.legendre = 1;
        return;
    }
    make_orbit_coeffs(o, coef);
    // Newton segment tables after the pieces (orbit_seg_offset, 16-byte aligned)
    int seg_nh = 0, seg_ng = 0, seg_div = 0, seg_a7 = 1;
    double seg_b6 = 0.0, seg_h6 = 0.0;
    coef.resize(orbit_table_doubles(o.n), 0.0);
    double* seg = coef.data() + orbit_seg_offset(o.n);
    make_orbit_segments(o, coef.data(), seg, seg_nh, seg_ng, seg_div, seg_a7, seg_b6, seg_h6);
    // their float pairs for the float-float Newton: b, h, g, a of each segment
    float2* ffs = reinterpret_cast<float2*>(coef.data() + orbit_segff_offset(o.n));
    auto split = [](double v) {
        const float hi = (float)v;
        return make_float2(hi, (float)(v - (double)hi));
    };
    for (int j = 0; j < o.n - 1; ++j) {
        const double* sj = seg + (size_t)j * SEG_STRIDE;
        float2* fj = ffs + (size_t)j * SEGFF_STRIDE;
        for (int k = 0; k < 21; ++k) fj[SEGFF_B + k] = split(sj[SEG_B + k]);
        for (int k = 0; k < SEG_NH; ++k) fj[SEGFF_H + k] = split(sj[SEG_H + k]);
        for (int k = 0; k < SEG_NG; ++k) fj[SEGFF_G + k] = split(sj[SEG_G + k]);
        for (int k = 0; k < 24; ++k) fj[SEGFF_A + k] = split(sj[SEG_A + k]);
    }
    ob = Orbit{};
    ob.t0 = o.t0;
    ob.spacing = o.spacing;
    ob.inv_spacing = 1.0 / o.spacing;
    ob.t_end = o.t0 + (o.n - 1) * o.spacing;
    ob.n = o.n;
    ob.n_pieces = o.n - 3;
    ob.seg_nh = seg_nh;
    ob.seg_ng = seg_ng;
    ob.seg_div = seg_div;
    ob.seg_a7 = seg_a7;
    ob.seg_b6 = seg_b6;
    ob.seg_h6 = seg_h6;
    ob.seg_r6 = 1;           // without a geometry to bound |D|: kept (residual_degree)
}

bool utm_setup(int code, Utm& u) {
    // core/Projections.cpp:80-170
    int zone;
    if (code > 32600 && code <= 32660) { zone = code - 32600; u.isnorth = 1; }
    else if (code > 32700 && code <= 32760) { zone = code - 32700; u.isnorth = 0; }
    else return false;
    u.lon0 = ((zone - 0.5) * (M_PI / 30.)) - M_PI;
    const double f = WGS84_E2 / (1. + std::sqrt(1 - WGS84_E2));
    const double n = f / (2. - f);
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
    const double Z = clens(u.cbg, 0.);
    u.Zb = -u.Qn * (Z + clens(u.gtu, 2 * Z));
    u.slon0 = std::sin(u.lon0);
    u.clon0 = std::cos(u.lon0);
    return true;
}

bool is_lonlat_or_utm(int epsg) { return epsg == 4326 || (epsg > 32600 && epsg <= 32660) || (epsg > 32700 && epsg <= 32760); }

// Map <-> lon/lat(rad) for LonLat or UTM (core/Projections.h:127-140).
bool proj_inverse(int epsg, const Utm& u, double x, double y, double& lon, double& lat) {
    if (epsg == 4326) { lon = x * M_PI / 180.0; lat = y * M_PI / 180.0; return true; }
    return utm_inverse(u, x, y, lon, lat);
}
bool proj_forward(int epsg, const Utm& u, double lon, double lat, double& x, double& y) {
    if (epsg == 4326) { x = lon * 180.0 / M_PI; y = lat * 180.0 / M_PI; return true; }
    return utm_forward(u, lon, lat, x, y);
}

// build_orbit_table through the context's cache of the last 16 orbits: a
// caller that geocodes many blocks, bands or requests with a few orbits
// builds their polynomial pieces and Newton tables once each (about 0.7 ms
// for 21 state vectors).  The key is the descriptor's scalars and the state
// vectors' bytes, so any change rebuilds.
constexpr size_t ORBIT_CACHE_ENTRIES = 16;
void orbit_table_cached(gslc_ctx* c, const gslc_orbit& o, std::vector<double>& coef, Orbit& ob) {
    const size_t nv = 3 * (size_t)o.n;
    const double head[4] = {o.t0, o.spacing, (double)o.n, (double)o.method};
    auto& cache = c->orbit_cache;
    size_t i = 0;
    for (; i < cache.size(); ++i) {
        const std::vector<double>& k = cache[i].key;
        if (k.size() == 4 + 2 * nv && std::memcmp(k.data(), head, sizeof(head)) == 0 &&
            std::memcmp(k.data() + 4, o.pos, nv * sizeof(double)) == 0 &&
            std::memcmp(k.data() + 4 + nv, o.vel, nv * sizeof(double)) == 0)
            break;
    }
    if (i == cache.size()) {
        gslc_ctx::OrbitTables t;
        build_orbit_table(o, t.coef, t.ob);
        t.key.assign(head, head + 4);
        t.key.insert(t.key.end(), o.pos, o.pos + nv);
        t.key.insert(t.key.end(), o.vel, o.vel + nv);
        if (cache.size() == ORBIT_CACHE_ENTRIES) cache.pop_back();
        cache.insert(cache.begin(), std::move(t));
    } else if (i > 0) {
        std::rotate(cache.begin(), cache.begin() + i, cache.begin() + i + 1);   // most recent first
    }
    coef = cache.front().coef;
    ob = cache.front().ob;
}

// The Newton residual's degree for ground points seen from the radar grid
// rg: the degree-6 term is dropped where it moves a step by less than
// 1e-12 s.  With |D| = |xyz - P_ref| at most the grid's far slant range
// plus half a segment of travel (10 km/s bounds the speed), the returned
// iterate then moves by < 1e-12 s, a tenth of the reference's own
// orbit-interpolation rounding (~1e-11 s), and the slant range, stationary
// at zero Doppler, does not move to first order.  Terms of H above degree 5
// (seg_nh >= 6) keep it.
int residual_degree6(const Orbit& ob, const gslc_radar_grid& rg) {
    if (ob.legendre) return 1;
    if (ob.seg_nh >= 6) return 1;
    const double far = rg.starting_range + std::max<int64_t>(rg.width - 1, 0) * rg.range_pixel_spacing;
    const double dmax = std::fabs(far) + 1e4 * 0.5 * ob.spacing;
    return dmax * ob.seg_b6 + ob.seg_h6 >= 1e-12 ? 1 : 0;
}

// Orbit descriptor checks: Hermite (4 or more state vectors) or Legendre
// (9 or more, core/detail/InterpolateOrbit.icc:111-155); uniform spacing.
int check_orbit(gslc_ctx* c, const gslc_orbit& o) {
    if (o.method != 0 && o.method != 1) return set_err(c, GSLC_EINVAL, "orbit interpolation method must be 0 or 1");
    if (o.n < 4 || !o.pos || !o.vel || !(o.spacing > 0))
        return set_err(c, GSLC_EINVAL, "orbit needs >= 4 uniformly spaced state vectors");
    if (o.method == 1 && o.n < 9)
        return set_err(c, GSLC_EINVAL, "Legendre orbit interpolation needs >= 9 state vectors");
    return GSLC_OK;
}

Lut to_lut(const gslc_lut2d& l, const double* sinc64 = nullptr) {
    Lut o{};
    o.have_data = l.have_data;
    o.bounds_error = l.bounds_error;
    o.method = l.method;
    o.nx = l.nx;
    o.ny = l.ny;
    o.x0 = l.x0; o.y0 = l.y0; o.dx = l.dx; o.dy = l.dy;
    o.ref_value = l.ref_value;
    o.inv_dx = 1.0 / l.dx;
    o.inv_dy = 1.0 / l.dy;
    lut_axis_keys(l.x0, l.dx, l.nx, o.kx_lo, o.kx_hi);
    lut_axis_keys(l.y0, l.dy, l.ny, o.ky_lo, o.ky_hi);
    o.data = l.data;
    o.sinc = sinc64;
    return o;
}

// The sinc kernel table in double on the device (a LUT2d with the sinc
// method, the raster interpolators), made on first use.
int ensure_sinc64(gslc_ctx* c) {
    if (c->d_sinc64) return GSLC_OK;
    if (c->no_alloc) return set_err(c, GSLC_EUNSUPPORTED, "a sinc LUT2d needs the context's sinc table");
    const std::vector<double> t = make_sinc_table_double();
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_sinc64, t.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_sinc64, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (c->d_sinc64) cudaFree(c->d_sinc64);
        c->d_sinc64 = nullptr;
        return cuda_err(c, e, "sinc table");
    }
    return GSLC_OK;
}

// LUT2d interpolation methods (isce3 dataInterpMethod): 0 sinc, 1 bilinear,
// 2 bicubic, 3 nearest, 4 biquintic
int check_lut(gslc_ctx* c, const gslc_lut2d& l, const char* name) {
    if (!l.have_data) return 0;
    if (l.method < 0 || l.method > 4)
        return set_err(c, GSLC_EINVAL, std::string(name) + ": unknown LUT2d interpolation method");
    if (l.nx < 1 || l.ny < 1 || !l.data) return set_err(c, GSLC_EINVAL, std::string(name) + ": LUT2d without data");
    if (l.method == 0) return ensure_sinc64(c);
    return 0;
}

int to_azrg(gslc_ctx* c, const gslc_azrg_func& f, AzRg& o, const char* name) {
    std::memset(&o, 0, sizeof(o));
    o.kind = f.kind;
    if (f.kind == 0) {
        if (int st = check_lut(c, f.lut, name)) return st;
        o.lut = to_lut(f.lut, c->d_sinc64);
        o.is_zero = (!f.lut.have_data && f.lut.ref_value == 0.0) ? 1 : 0;
    } else if (f.kind == 1) {
        const gslc_poly2d& p = f.poly;
        const int nc = (p.x_order + 1) * (p.y_order + 1);
        if (p.x_order < -1 || p.y_order < -1) return set_err(c, GSLC_EINVAL, std::string(name) + ": bad Poly2d order");
        if (nc > POLY_MAX) return set_err(c, GSLC_EUNSUPPORTED, std::string(name) + ": Poly2d has more than 64 coefficients");
        o.poly.x_order = p.x_order;
        o.poly.y_order = p.y_order;
        o.poly.x_mean = p.x_mean; o.poly.y_mean = p.y_mean;
        o.poly.x_norm = p.x_norm; o.poly.y_norm = p.y_norm;
        o.poly.inv_x_norm = 1.0 / p.x_norm;
        o.poly.inv_y_norm = 1.0 / p.y_norm;
        for (int i = 0; i < nc; ++i) o.poly.c[i] = p.coeffs[i];
        // the default Poly2d (order -1) evaluates to exactly 0 (core/Poly2d.h:56)
        o.is_zero = nc <= 0 ? 1 : 0;
    } else {
        return set_err(c, GSLC_EINVAL, std::string(name) + ": unknown carrier kind");
    }
    return 0;
}

}  // namespace

// ---- DEM window: geometry/loadDem.cpp:22-133 + DEMInterpolator.cpp:29-455 --
extern "C" int gslc_compute_dem_window(const gslc_dem_raster* r, const gslc_geo_grid* g, int32_t margin, gslc_dem_window* out) {
    if (!r || !g || !out) return GSLC_EINVAL;
    return gslc_compute_dem_window_block(r, g, 0, g->length, g->width, margin, out);
}

extern "C" int gslc_compute_dem_window_block(const gslc_dem_raster* r, const gslc_geo_grid* g, int32_t line_start,
                                             int32_t block_length, int32_t block_width, int32_t margin,
                                             gslc_dem_window* out) {
    if (!r || !g || !out) return GSLC_EINVAL;
    std::memset(out, 0, sizeof(*out));
    if (!is_lonlat_or_utm(r->epsg) || !is_lonlat_or_utm(g->epsg)) return GSLC_EUNSUPPORTED;
    if (r->gt[2] != 0.0 || r->gt[4] != 0.0) return GSLC_EUNSUPPORTED;
    const int lineStart = line_start, blockLength = block_length, blockWidth = block_width;
    double minX = std::numeric_limits<double>::max(), maxX = std::numeric_limits<double>::lowest();
    double minY = std::numeric_limits<double>::max(), maxY = std::numeric_limits<double>::lowest();
    if (r->epsg != g->epsg) {
        Utm ug{}, ud{};
        if (g->epsg != 4326) utm_setup(g->epsg, ug);
        if (r->epsg != 4326) utm_setup(r->epsg, ud);
        const int askip = std::max(static_cast<int>(blockLength / 10.), 1);
        const int rskip = std::max(static_cast<int>(blockWidth / 10.), 1);
        std::vector<int> li, pi;
        for (int j = 0; j < blockWidth; j += rskip) { li.push_back(0); pi.push_back(j); }
        for (int i = 0; i < blockLength; i += askip) { li.push_back(i); pi.push_back(blockWidth); }
        for (int j = blockWidth; j > 0; j -= rskip) { li.push_back(blockLength - 1); pi.push_back(j); }
        for (int i = blockLength; i > 0; i -= askip) { li.push_back(i); pi.push_back(0); }
        for (size_t i = 0; i < li.size(); ++i) {
            const double ox = g->start_x + g->spacing_x * pi[i];
            const double oy = g->start_y + g->spacing_y * (lineStart + li[i]);
            double lon, lat, dx, dy;
            if (!proj_inverse(g->epsg, ug, ox, oy, lon, lat) || !proj_forward(r->epsg, ud, lon, lat, dx, dy))
                return GSLC_EPROJ;
            minX = std::min(minX, dx); maxX = std::max(maxX, dx);
            minY = std::min(minY, dy); maxY = std::max(maxY, dy);
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

    // DEMInterpolator::loadDEM
    double min_x = minX, max_x = maxX, min_y = minY, max_y = maxY;
    const double delta_y = r->gt[5], delta_x = r->gt[1];
    // a negative x spacing makes loadDEM warn and return InvalidDem; the
    // interpolator then has no raster and yields the reference height
    // (DEMInterpolator.cpp:43-49)
    if (delta_x < 0) return GSLC_OK;
    const double dem_y0 = r->gt[3];
    double dem_x0 = r->gt[0];
    const bool ll = r->epsg == 4326;
    if (ll) {
        if (max_x - min_x > 360 + 2 * delta_x) max_x = min_x + 360 + delta_x;
        if (min_x < -180 - delta_x || max_x < -180 - delta_x || max_x > 360 + delta_x) {
            const double n_wraps = std::floor(max_x / 360);
            min_x -= n_wraps * 360;
            max_x -= n_wraps * 360;
        }
        if (min_x < -180 - delta_x || max_x < -180 - delta_x) { min_x += 360; max_x += 360; }
        if (min_x > 0 && max_x < 0) max_x += 360;
        if (dem_x0 > 360 + delta_x || dem_x0 < -180 - delta_x) dem_x0 = std::fmod(dem_x0, 360);
    }
    const double dem_yf = dem_y0 + r->length * delta_y;
    const double dem_xf = dem_x0 + r->width * delta_x;
    if (ll && min_x < dem_xf - 360 - delta_x) { min_x += 360; max_x += 360; }
    else if (ll && min_x > 180 && max_x > dem_x0 + 360 + delta_x) { min_x -= 360; max_x -= 360; }
    const bool disc = ll && (min_x <= dem_xf) && (dem_xf < max_x) && (min_x <= dem_x0 + 360) && (dem_x0 + 360 < max_x);
    if (min_x < dem_x0) min_x = dem_x0;
    if (max_x > dem_xf && !disc) max_x = dem_xf;
    if (min_y < dem_yf) min_y = dem_yf;
    if (max_y > dem_y0) max_y = dem_y0;
    long min_x_idx = (long)std::floor((min_x - dem_x0) / delta_x);
    long max_x_idx = (long)std::ceil((max_x - dem_x0) / delta_x);
    long min_y_idx = (long)std::floor((max_y - dem_y0) / delta_y);
    long max_y_idx = (long)std::ceil((min_y - dem_y0) / delta_y);
    out->x_start = dem_x0 + (0.5 + min_x_idx) * delta_x;
    out->y_start = dem_y0 + (0.5 + min_y_idx) * delta_y;
    out->dx = delta_x;
    out->dy = delta_y;
    long width = max_x_idx - min_x_idx, length = max_y_idx - min_y_idx;
    if (!disc && min_x_idx + width > r->width) width = r->width - min_x_idx;
    if (!disc && min_y_idx + length > r->length) length = r->length - min_y_idx;
    out->x_off = min_x_idx;
    out->y_off = min_y_idx;
    out->width = width;
    out->length = length;
    out->wraps = disc ? 1 : 0;
    // A window with no pixels leaves the interpolator without a raster: every
    // height is then the reference height (DEMInterpolator.cpp:393-397).
    out->have_raster = (width > 0 && length > 0) ? 1 : 0;
    if (out->have_raster && (min_x_idx < 0 || min_y_idx < 0)) return GSLC_EINVAL;
    return GSLC_OK;
}

extern "C" int gslc_orbit_interpolate(const gslc_orbit* o, double t, double* pos, double* vel) {
    if (!o || !pos || !vel || o->n < 4 || !(o->spacing > 0) || (o->method != 0 && o->method != 1) ||
        (o->method == 1 && o->n < 9) || !o->pos || !o->vel)
        return GSLC_EINVAL;
    std::vector<double> coef;
    Orbit ob{};
    if (o->method == 1) {
        build_orbit_table(*o, coef, ob);
    } else {
        make_orbit_coeffs(*o, coef);
        ob.t0 = o->t0; ob.spacing = o->spacing; ob.inv_spacing = 1.0 / o->spacing;
        ob.t_end = o->t0 + (o->n - 1) * o->spacing; ob.n = o->n; ob.n_pieces = o->n - 3;
    }
    ob.coef = coef.data();
    if (!(t >= ob.t0 && t <= ob.t_end)) return GSLC_EINVAL;
    V3 p, v;
    orbit_eval(ob, t, p, v);
    pos[0] = p.x; pos[1] = p.y; pos[2] = p.z;
    vel[0] = v.x; vel[1] = v.y; vel[2] = v.z;
    return GSLC_OK;
}

extern "C" int gslc_geo2rdr_zero_doppler(const gslc_orbit* o, const double* xyz, double t_guess, int32_t look_side,
                                         double threshold, int32_t maxiter, double* aztime, double* slant_range,
                                         int32_t* converged) {
    if (!o || !xyz || !aztime || !slant_range || !converged || o->n < 4 || !(o->spacing > 0) ||
        (o->method != 0 && o->method != 1) || (o->method == 1 && o->n < 9) || !o->pos || !o->vel ||
        (look_side != -1 && look_side != 1))
        return GSLC_EINVAL;
    std::vector<double> coef;
    Orbit ob;
    build_orbit_table(*o, coef, ob);
    ob.coef = coef.data();
    ob.seg_ff = reinterpret_cast<const float2*>(coef.data() + orbit_segff_offset(ob.n));
    ob.seg = coef.data() + orbit_seg_offset(o->n);
    *converged = 0;
    *aztime = *slant_range = std::nan("");
    // iteration 0 (geometry/detail/Geo2Rdr.icc:114-179): look side and first step at t_guess
    if (!(t_guess >= ob.t0 && t_guess <= ob.t_end)) return GSLC_OK;
    if (maxiter < 1) return GSLC_OK;
    const V3 x{xyz[0], xyz[1], xyz[2]};
    V3 pos, vel;
    orbit_eval(ob, t_guess, pos, vel);
    const V3 rvec = vsub(x, pos);
    // the kernels' form of iteration 0 (look side and step from per-launch constants)
    if ((look_side == -1) != (vdot(rvec, vcross(vel, pos)) > 0.)) return GSLC_OK;
    double t = t_guess, R = 0.0;
    const double dt = -vdot(rvec, vel) * (1.0 / vdot(vel, vel));
    bool ok;
    if (std::fabs(dt) < threshold) {
        R = vnorm(rvec);
        ok = true;
    } else {
        ok = ob.legendre ? geo2rdr_zero_doppler_orbit(ob, x, threshold, maxiter, t, dt, R)
                         : geo2rdr_zero_doppler_seg(ob, ob.seg, x, threshold, maxiter, t, dt, R);
    }
    if (ok) {
        *aztime = t;
        *slant_range = R;
        *converged = 1;
    }
    return GSLC_OK;
}

extern "C" int gslc_sinc_table(float* out) {
    if (!out) return GSLC_EINVAL;
    const std::vector<float> t = make_sinc_table();
    std::memcpy(out, t.data(), t.size() * sizeof(float));
    return GSLC_OK;
}

extern "C" const char* gslc_version(void) { return "gslc 0.1 (sm_103a)"; }

extern "C" int gslc_ctx_create(int device, gslc_ctx** out) {
    if (!out) return GSLC_EINVAL;
    *out = nullptr;
    gslc_ctx* c = new (std::nothrow) gslc_ctx();
    if (!c) return GSLC_ECUDA;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete c; return GSLC_ECUDA; }
    const std::vector<float> table = make_sinc_table();
    e = cudaMalloc(&c->d_sinc, table.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_sinc, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_err, sizeof(int32_t) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_err, sizeof(int32_t) * 4);
    if (e != cudaSuccess) { gslc_ctx_destroy(c); return GSLC_ECUDA; }
    // The calls' scratch (deramped copies, batch buffers, planner and cube
    // scratch) is stream-ordered memory of the device's default pool.  With
    // the pool's default release threshold of 0 every synchronisation hands
    // it back to the driver and the next call maps it again; keep up to
    // 16 GiB cached instead (process-local; a higher threshold is kept).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t cur = 0, keep = 16ull << 30;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur) == cudaSuccess && cur < keep)
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    *out = c;
    return GSLC_OK;
}

extern "C" int gslc_ctx_destroy(gslc_ctx* c) {
    if (!c) return GSLC_OK;
    cudaSetDevice(c->device);
    if (c->d_sinc) cudaFree(c->d_sinc);
    if (c->d_err) cudaFree(c->d_err);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->d_orbit) cudaFree(c->d_orbit);
    if (c->d_sinc64) cudaFree(c->d_sinc64);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->band_ev)
        if (e) cudaEventDestroy(e);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    for (auto& e : c->io_ev)
        if (e) cudaEventDestroy(e);
    if (c->h2d_stream) cudaStreamDestroy(c->h2d_stream);
    if (c->aux_stream) cudaStreamDestroy(c->aux_stream);
    delete c;
    return GSLC_OK;
}

extern "C" const char* gslc_last_error(const gslc_ctx* c) { return c ? c->err.c_str() : "no context"; }
extern "C" int64_t gslc_last_launch_count(const gslc_ctx* c) { return c ? c->launches : 0; }

namespace {

bool grid_ok(const gslc_radar_grid& g) {
    return g.prf > 0 && g.range_pixel_spacing != 0 && g.length > 0 && g.width > 0 && g.wavelength > 0 &&
           (g.look_side == -1 || g.look_side == 1);
}
double grid_stop(const gslc_radar_grid& g) { return g.sensing_start + (g.length - 1.0) / g.prf; }
double grid_end(const gslc_radar_grid& g) { return g.starting_range + (g.width - 1.0) * g.range_pixel_spacing; }

}  // namespace

namespace {

// The kernel's view of a DEM window: samples, size and pixel-centre start
// (DEMInterpolator fields after loadDEM), checked against the samples given.
int bind_dem_window(gslc_ctx* c, const gslc_dem_raster& d, const gslc_dem_window& w, Dem& dem) {
    dem.have_raster = w.have_raster && d.data != nullptr;
    dem.epsg_is_lonlat = d.epsg == 4326;
    if (!dem.epsg_is_lonlat) utm_setup(d.epsg, dem.utm);
    if (dem.have_raster) {
        if (w.x_off < d.data_x_off || w.y_off < d.data_y_off || w.x_off + w.width > d.data_x_off + d.data_width ||
            w.y_off + w.length > d.data_y_off + d.data_length || d.data_stride < d.data_width)
            return set_err(c, GSLC_EINVAL, "DEM samples provided do not cover the DEM window of the geogrid");
        dem.data = d.data + (w.y_off - d.data_y_off) * d.data_stride + (w.x_off - d.data_x_off);
        dem.stride = d.data_stride;
        dem.width = (int32_t)w.width;
        dem.length = (int32_t)w.length;
        dem.x_start = w.x_start; dem.y_start = w.y_start;
        dem.dx = w.dx; dem.dy = w.dy;
    }
    dem.sc = make_spline_const();
    dem.avail_lo = 0;
    dem.avail_hi = INT32_MAX;
    dem.err = nullptr;
    return GSLC_OK;
}

// Validation and launch parameters of one geocode call: everything except
// the device addresses of the orbit polynomials (bind_orbit), the sinc table
// and the error word.  GSLC_EMPTY_GRID means there is nothing to do.
constexpr int GSLC_EMPTY_GRID = 100;
// The sinc chip's native Doppler from the radar indices (GeoParams::chip_dop):
// the reference's contains(az, rng) at az = t0 + azc / prf and
// rng = r0 + rgc * dr (geocodeSlc.cpp:457-467), monotone in each index, as
// key intervals of azc and rgc; the table's origin in radar indices and
// its cells per index for the FP32 coordinates.  Left off (the FP64 form)
// for other methods, tables without data, degenerate spacings, or tables
// spanning 2^21 radar lines or samples or more.
void chip_doppler(GeoParams& p, const gslc_lut2d& l, const gslc_radar_grid& rg) {
    p.chip_dop = 0;
    if (!l.have_data || l.method != 1 || l.nx < 1 || l.ny < 1) return;
    const double prf = rg.prf, t0 = rg.sensing_start, dr = rg.range_pixel_spacing, r0 = rg.starting_range;
    for (double v : {prf, t0, dr, r0, l.x0, l.y0, l.dx, l.dy})
        if (!std::isfinite(v)) return;
    if (prf == 0.0 || dr == 0.0 || l.dx == 0.0 || l.dy == 0.0) return;
    const double saz = 1.0 / (prf * l.dy), srg = dr / l.dx;          // cells per line, per sample
    const double caz = (l.y0 - t0) * prf, crg = (l.x0 - r0) / dr;    // the table's first cell in radar indices
    const double lim = 2097152.0;                                    // 2^21
    if (!((l.ny - 1.0) / std::fabs(saz) < lim && (l.nx - 1.0) / std::fabs(srg) < lim)) return;
    if (!(std::fabs(caz) < 1e9 && std::fabs(crg) < 1e9)) return;
    const double y0 = l.y0, dy = l.dy, x0 = l.x0, dx = l.dx;
    key_interval([&](double azc) { return ((t0 + azc / prf) - y0) / dy; }, (prf > 0) == (dy > 0), l.ny - 1.0,
                 p.cd_kaz_lo, p.cd_kaz_hi);
    key_interval([&](double rgc) { return ((r0 + rgc * dr) - x0) / dx; }, (dr > 0) == (dx > 0), l.nx - 1.0,
                 p.cd_krg_lo, p.cd_krg_hi);
    const double iaz = std::floor(caz), irg = std::floor(crg);
    p.cd_iaz = (int32_t)iaz;
    p.cd_irg = (int32_t)irg;
    p.cd_faz = (float)(caz - iaz);
    p.cd_frg = (float)(crg - irg);
    p.cd_saz = (float)saz;
    p.cd_srg = (float)srg;
    p.chip_dop = 1;
}

int prepare_geocode(gslc_ctx* c, const gslc_geocode_args* a, GeoParams& p, std::vector<double>& coef) {
    if (!a) return set_err(c, GSLC_EINVAL, "null arguments");
    const gslc_radar_grid& rg = a->radar_grid;
    const gslc_radar_grid& srg = a->sliced_radar_grid;
    const gslc_geo_grid& gg = a->geo_grid;
    if (a->n_blocks < 1 || !a->rdr_blocks || !a->geo_blocks)
        return set_err(c, GSLC_EINVAL, "number of geoDataBlocks != number of rdrDataBlocks");
    if (!grid_ok(rg) || !grid_ok(srg)) return set_err(c, GSLC_EINVAL, "invalid radar grid");
    if (gg.width < 0 || gg.length < 0) return set_err(c, GSLC_EINVAL, "invalid geogrid");
    // geocodeSlc.cpp:548-580 (validate_slice)
    if (srg.sensing_start < rg.sensing_start) return set_err(c, GSLC_EINVAL, "sliced grid sensing start < full grid sensing start");
    if (grid_stop(srg) > grid_stop(rg)) return set_err(c, GSLC_EINVAL, "sliced grid sensing stop < full grid sensing stop");
    if (srg.starting_range < rg.starting_range) return set_err(c, GSLC_EINVAL, "sliced grid staring range < full grid staring range");
    if (grid_end(srg) > grid_end(rg)) return set_err(c, GSLC_EINVAL, "sliced grid ending range < full grid ending range");
    if (srg.look_side != rg.look_side) return set_err(c, GSLC_EINVAL, "sliced grid look side != full grid look side");
    if (srg.wavelength != rg.wavelength) return set_err(c, GSLC_EINVAL, "sliced grid wavelength != full grid wavelength");
    if (!is_lonlat_or_utm(gg.epsg)) return set_err(c, GSLC_EUNSUPPORTED, "geogrid EPSG must be 4326 or UTM");
    if (int st = check_orbit(c, a->orbit)) return st;
    if (a->rdr_length < 0 || a->rdr_width < 0) return set_err(c, GSLC_EINVAL, "invalid radar block shape");
    if (a->rdr_format != 0 && a->rdr_format != 1) return set_err(c, GSLC_EINVAL, "rdr_format must be 0 (complex64) or 1 (complex32)");
    if (a->geo_format < 0 || a->geo_format > 2) return set_err(c, GSLC_EINVAL, "geo_format must be 0, 1 or 2");
    if (a->geo_format == 2 && !(a->mantissa_bits > 0 && a->mantissa_bits <= 23))
        return set_err(c, GSLC_EINVAL, "Require 0 < significant_bits <= 23");
    if (a->rdr_format == 1 && a->inplace_deramp)
        return set_err(c, GSLC_EINVAL, "in-place deramp needs complex64 radar blocks");
    if (gg.width == 0 || gg.length == 0) return GSLC_EMPTY_GRID;
    for (const gslc_lut2d* l : {&a->native_doppler, &a->image_grid_doppler, &a->az_time_correction, &a->srange_correction})
        if (int st = check_lut(c, *l, "LUT2d")) return st;

    std::memset(&p, 0, sizeof(p));
    p.dop_dr = 1.0e-8;      // geocodeSlc.cpp:120-123
    p.gx0 = gg.start_x; p.gy0 = gg.start_y; p.gdx = gg.spacing_x; p.gdy = gg.spacing_y;
    p.gw = gg.width; p.gl = gg.length;
    p.geo_is_lonlat = gg.epsg == 4326;
    if (!p.geo_is_lonlat) utm_setup(gg.epsg, p.utm);
    p.tile_fit = p.geo_is_lonlat ? 0 : 1;
    p.rdr_c32 = a->rdr_format == 1 ? 1 : 0;
    p.geo_fmt = a->geo_format;
    p.mant_bits = a->geo_format == 2 ? a->mantissa_bits : 23;
    p.stage_wait = c && c->stage_wait > 0 ? c->stage_wait : STAGE_WAIT_DEFAULT;
    p.avail_az_lo = INT64_MIN / 2;
    p.avail_az_hi = INT64_MAX / 2;

    // DEM window the reference would load (loadDem.cpp:22-133)
    gslc_dem_window w;
    int st = gslc_compute_dem_window(&a->dem, &gg, a->dem_margin, &w);
    if (st == GSLC_EPROJ) return set_err(c, GSLC_EINVAL, "projection transformation between geogrid and DEM failed");
    if (st != GSLC_OK) return set_err(c, st, "unsupported or invalid DEM raster");
    if (w.wraps) return set_err(c, GSLC_EUNSUPPORTED, "DEM window crossing the DEM file discontinuity");
    if ((st = bind_dem_window(c, a->dem, w, p.dem))) return st;
    p.ell_a = a->ellipsoid_a;
    p.ell_e2 = a->ellipsoid_e2;

    // orbit polynomials and Newton tables
    orbit_table_cached(c, a->orbit, coef, p.orbit);
    p.orbit.seg_r6 = residual_degree6(p.orbit, a->radar_grid);
    const Orbit& ob = p.orbit;

    // geo2rdr setup: initial guess sensingMid (geocodeSlc.cpp:108)
    p.t_mid = 0.5 * (rg.sensing_start + grid_stop(rg));
    p.t_mid_in_orbit = (p.t_mid >= ob.t0 && p.t_mid <= ob.t_end) ? 1 : 0;
    if (p.t_mid_in_orbit) {
        Orbit host_ob = ob;
        host_ob.coef = coef.data();
        orbit_eval(host_ob, p.t_mid, p.pos0, p.vel0);
        p.n0 = vcross(p.vel0, p.pos0);
        p.inv_vv0 = 1.0 / vdot(p.vel0, p.vel0);
    }
    p.thr = a->threshold_geo2rdr;
    p.thr_bits = p.thr > 0.0 ? dbits(p.thr) : 0ull;
    p.maxiter = a->numiter_geo2rdr;
    p.rg_t0 = rg.sensing_start; p.rg_prf = rg.prf; p.rg_r0 = rg.starting_range;
    p.rg_dr = rg.range_pixel_spacing; p.rg_wvl = rg.wavelength;
    p.rg_inv_dr = 1.0 / p.rg_dr;
    p.rg_len = rg.length; p.rg_wid = rg.width;
    p.look_side = rg.look_side;
    // sliced grid contains() bounds (RadarGridParameters.cpp:27-35)
    const double half_az = (1.0 / srg.prf) / 2, half_rg = srg.range_pixel_spacing / 2;
    p.s_t0 = srg.sensing_start - half_az;
    p.s_r0 = srg.starting_range - half_rg;
    p.s_stop = grid_stop(srg) + half_az;
    p.s_end = grid_end(srg) + half_rg;
    p.k_s_t0 = dkey(p.s_t0);
    p.k_s_stop = dkey(p.s_stop);
    p.k_s_r0 = dkey(p.s_r0);
    p.k_s_end = dkey(p.s_end);
    p.nat_dop = to_lut(a->native_doppler, c->d_sinc64);
    chip_doppler(p, a->native_doppler, rg);
    p.img_dop = to_lut(a->image_grid_doppler, c->d_sinc64);
    p.az_corr = to_lut(a->az_time_correction, c->d_sinc64);
    p.sr_corr = to_lut(a->srange_correction, c->d_sinc64);
    p.az_corr_on = p.az_corr.have_data || p.az_corr.ref_value != 0.0;
    p.sr_corr_on = p.sr_corr.have_data || p.sr_corr.ref_value != 0.0;
    if ((st = to_azrg(c, a->az_carrier, p.az_car, "az_carrier"))) return st;
    if ((st = to_azrg(c, a->rg_carrier, p.rg_car, "rg_carrier"))) return st;
    p.carriers_zero = p.az_car.is_zero && p.rg_car.is_zero;
    p.flat_scale = 4.0 * (M_PI / rg.wavelength);
    p.inv_prf = 1.0 / rg.prf;
    p.two_pi_over_prf = 2.0 * M_PI / rg.prf;
    p.two_pi_over_prf_f = (float)p.two_pi_over_prf;
    p.flatten = a->flatten; p.reramp = a->reramp; p.use_corr = a->flatten_with_corrected_srange;
    p.inv_re = a->invalid_re; p.inv_im = a->invalid_im;
    p.inL = a->rdr_length; p.inW = a->rdr_width;
    p.az_first = a->first_azimuth_line; p.rg_first = a->first_range_sample;
    p.az_first_d = (double)p.az_first;
    p.rg_first_d = (double)p.rg_first;
    p.mask = a->mask;
    p.carrier_out = a->carrier_phase;
    p.flatten_out = a->flatten_phase;
    p.az_out = a->az_index;
    p.rg_out = a->rg_index;
    if (a->subswaths) {
        p.have_subsw = 1;
        p.subsw_n = a->subswaths->n;
        p.subsw_len = a->subswaths->length;
        p.subsw_wid = a->subswaths->width;
        p.subsw = a->subswaths->valid;
        if (p.subsw_n > 0 && !p.subsw) return set_err(c, GSLC_EINVAL, "subswaths without valid-sample arrays");
    }
    return GSLC_OK;
}

// Point the launch parameters at orbit polynomials resident at d_coef
// (doubles, then the float pairs, as make_orbit_coeffs + prepare lay them out).
void bind_orbit(GeoParams& p, const double* d_coef) {
    p.orbit.coef = d_coef;
    p.orbit.seg_ff = reinterpret_cast<const float2*>(d_coef + orbit_segff_offset(p.orbit.n));
    p.orbit.seg = d_coef + orbit_seg_offset(p.orbit.n);
}

}  // namespace

namespace {

// bytes per output pixel of the geo blocks in format f (gslc_geocode_args.geo_format)
size_t geo_pixel_bytes(int f) { return f == 1 ? 4 : 8; }

// gslc_geocode_slc, and with host_geo set the copies of the geo blocks (and
// of the mask, with host_mask) to host memory: the geogrid runs in row bands
// whose boundaries are multiples of every tile height (so every tile, and
// every pixel's value, is the one of the single launch), each band's copies
// queued on the context's copy stream behind its kernels.  deramp_buf, when
// given, receives the deramped copies of the radar blocks (block b at
// b * rdr_length * rdr_width, complex64) in place of stream-ordered scratch.
// lines_per_block > 0 is the raster mode (geocode/geocodeSlc.cpp:605-828):
// the geogrid runs in blocks of that many lines, each with its own DEM
// window (DEMRasterToInterpolator of the block, :653-656), and the phase
// outputs start as the invalid value's real part (:713-723).  The reference
// reads each block's radar bounding box widened by 5 samples (:740-750);
// the interpolator's chip tests then reject exactly the pixels they reject
// on the whole radar raster (the box is clamped only at the raster's edges),
// so the whole raster, deramped once, is read here.
int geocode_slc_impl(gslc_ctx* c, const gslc_geocode_args* a, cudaStream_t stream, void* const* host_geo,
                     uint8_t* host_mask, float2* deramp_buf = nullptr, int32_t lines_per_block = 0) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    GeoParams p;
    std::vector<double> coef;
    int st = prepare_geocode(c, a, p, coef);
    if (st == GSLC_EMPTY_GRID) return GSLC_OK;
    if (st != GSLC_OK) return st;
    const gslc_radar_grid& rg = a->radar_grid;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    if (coef.size() > c->orbit_cap) {
        if (c->d_orbit) cudaFree(c->d_orbit);
        c->d_orbit = nullptr;
        e = cudaMalloc(&c->d_orbit, coef.size() * sizeof(double));
        if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc orbit");
        c->orbit_cap = coef.size();
    }
    e = cudaMemcpyAsync(c->d_orbit, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cuda_err(c, e, "orbit upload");
    bind_orbit(p, c->d_orbit);
    p.sinc = c->d_sinc;
    p.err = c->d_err;
    e = cudaMemsetAsync(c->d_err, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return cuda_err(c, e, "memset");

    // carrier deramp: the reference mutates the radar blocks in place
    // (geocodeSlc.cpp:952-953); without inplace_deramp the deramped copy goes
    // to stream-ordered scratch.
    const int64_t nrdr = a->rdr_length * a->rdr_width;
    std::vector<void*> scratch;
    // every failure after this point: hand back the scratch, and let copies
    // already queued to the caller's host buffers finish before returning
    auto fail = [&](int code) {
        for (void* s : scratch) cudaFreeAsync(s, stream);
        if (host_geo && c->copy_stream) cudaStreamSynchronize(c->copy_stream);
        return code;
    };
    std::vector<const float2*> rdr(a->n_blocks);
    for (int b = 0; b < a->n_blocks; ++b) rdr[b] = (const float2*)a->rdr_blocks[b];
    if (c->timing) cudaEventRecord(c->ev[2], stream);
    if (!p.carriers_zero && nrdr > 0 && !a->rdr_deramped) {
        for (int b = 0; b < a->n_blocks; ++b) {
            float2* dst = (float2*)a->rdr_blocks[b];
            if (a->inplace_deramp) {
                // the caller's block (the reference's behaviour)
            } else if (deramp_buf) {
                dst = deramp_buf + (int64_t)b * nrdr;
            } else {
                void* buf = nullptr;
                e = cudaMallocAsync(&buf, nrdr * sizeof(float2), stream);
                if (e != cudaSuccess) return fail(cuda_err(c, e, "cudaMallocAsync deramp scratch"));
                scratch.push_back(buf);
                dst = (float2*)buf;
            }
            DerampParams dp;
            std::memset(&dp, 0, sizeof(dp));
            dp.src = rdr[b]; dp.dst = dst;
            dp.src_c32 = p.rdr_c32;
            dp.inL = a->rdr_length; dp.inW = a->rdr_width;
            dp.az_first = a->first_azimuth_line; dp.rg_first = a->first_range_sample;
            dp.rg_t0 = rg.sensing_start; dp.rg_prf = rg.prf; dp.rg_r0 = rg.starting_range; dp.rg_dr = rg.range_pixel_spacing;
            dp.inv_prf = 1.0 / rg.prf;
            dp.az_car = p.az_car; dp.rg_car = p.rg_car;
            e = launch_deramp(dp, stream, &c->launches);
            if (e != cudaSuccess) return fail(cuda_err(c, e, "deramp launch"));
            rdr[b] = dst;
        }
        p.rdr_c32 = 0;      // the deramped copies are complex64
    }
    if (c->timing) {
        cudaEventRecord(c->ev[3], stream);
        cudaEventRecord(c->ev[0], stream);
    }
    const int64_t gl = p.gl, gw = p.gw;
    int nband = 1;
    int64_t band_rows = gl;
    if (lines_per_block > 0) {
        band_rows = lines_per_block;
        nband = (int)((gl + band_rows - 1) / band_rows);
        const double fill = (double)a->invalid_re;
        for (double* ph : {a->carrier_phase, a->flatten_phase})
            if (ph && (e = launch_fill_f64(ph, gl * gw, fill, stream, &c->launches)) != cudaSuccess)
                return fail(cuda_err(c, e, "phase fill"));
    } else if (host_geo) {
        if (!c->copy_stream) {
            e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
            if (e != cudaSuccess) { c->copy_stream = nullptr; return fail(cuda_err(c, e, "copy stream")); }
        }
        for (auto& ev : c->band_ev)
            if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) {
                ev = nullptr;
                return fail(cuda_err(c, e, "band event"));
            }
        band_rows = ((gl + GSLC_HOST_BANDS - 1) / GSLC_HOST_BANDS + 31) / 32 * 32;
        nband = (int)((gl + band_rows - 1) / band_rows);
    }
    const size_t esz = geo_pixel_bytes(a->geo_format);
    for (int band = 0; band < nband; ++band) {
        const int64_t row0 = (int64_t)band * band_rows;
        const int64_t rows = std::min(band_rows, gl - row0);
        const int64_t off = row0 * gw;
        p.geo_row0 = row0;
        p.gl = rows;
        if (lines_per_block > 0) {
            gslc_dem_window w;
            const gslc_geo_grid& gg = a->geo_grid;
            int st = gslc_compute_dem_window_block(&a->dem, &gg, (int32_t)row0, (int32_t)rows, gg.width, a->dem_margin, &w);
            if (st == GSLC_EPROJ) st = set_err(c, GSLC_EINVAL, "projection transformation between geogrid and DEM failed");
            else if (st != GSLC_OK) st = set_err(c, st, "unsupported or invalid DEM raster");
            else if (w.wraps) st = set_err(c, GSLC_EUNSUPPORTED, "DEM window crossing the DEM file discontinuity");
            else st = bind_dem_window(c, a->dem, w, p.dem);
            if (st != GSLC_OK) return fail(st);
        }
        p.mask = a->mask ? a->mask + off : nullptr;
        p.carrier_out = a->carrier_phase ? a->carrier_phase + off : nullptr;
        p.flatten_out = a->flatten_phase ? a->flatten_phase + off : nullptr;
        p.az_out = a->az_index ? a->az_index + off : nullptr;
        p.rg_out = a->rg_index ? a->rg_index + off : nullptr;
        for (int b0 = 0; b0 < a->n_blocks; b0 += MAX_BLOCKS) {
            p.nblk = std::min(MAX_BLOCKS, a->n_blocks - b0);
            for (int b = 0; b < p.nblk; ++b) {
                p.rdr[b] = rdr[b0 + b];
                p.geo[b] = (float2*)((char*)a->geo_blocks[b0 + b] + off * esz);
            }
            e = launch_geocode(p, a->geo2rdr_precision, stream, &c->launches);
            if (e != cudaSuccess) return fail(cuda_err(c, e, "geocode launch"));
        }
        if (!host_geo) continue;
        e = cudaEventRecord(c->band_ev[band], stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->band_ev[band], 0);
        for (int b = 0; b < a->n_blocks && e == cudaSuccess; ++b)
            e = cudaMemcpyAsync((char*)host_geo[b] + off * esz, (const char*)a->geo_blocks[b] + off * esz,
                                (size_t)(rows * gw) * esz, cudaMemcpyDeviceToHost, c->copy_stream);
        if (e == cudaSuccess && host_mask && a->mask)
            e = cudaMemcpyAsync(host_mask + off, a->mask + off, (size_t)(rows * gw), cudaMemcpyDeviceToHost,
                                c->copy_stream);
        if (e != cudaSuccess) return fail(cuda_err(c, e, "band copy"));
    }
    if (host_geo) {
        e = cudaEventRecord(c->band_ev[GSLC_HOST_BANDS], c->copy_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, c->band_ev[GSLC_HOST_BANDS], 0);
        if (e != cudaSuccess) return fail(cuda_err(c, e, "band copy"));
    }
    if (c->timing) cudaEventRecord(c->ev[1], stream);
    for (void* s : scratch) cudaFreeAsync(s, stream);
    e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_err(c, e, "geocode");
    if (c->timing) {
        cudaEventElapsedTime(&c->ms_geocode, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&c->ms_deramp, c->ev[2], c->ev[3]);
    }
    return device_status(c, c->h_err[0]);
}

}  // namespace

extern "C" int gslc_geocode_slc(gslc_ctx* c, const gslc_geocode_args* a, void* stream) {
    return geocode_slc_impl(c, a, (cudaStream_t)stream, nullptr, nullptr);
}

extern "C" int gslc_geocode_slc_raster(gslc_ctx* c, const gslc_geocode_args* a, int32_t lines_per_block,
                                       void* stream) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    if (!a) return set_err(c, GSLC_EINVAL, "null arguments");
    if (lines_per_block < 1) return set_err(c, GSLC_EINVAL, "lines_per_block must be positive");
    if (a->rdr_length != a->radar_grid.length || a->rdr_width != a->radar_grid.width)
        return set_err(c, GSLC_EINVAL, "input raster shape differs from the radar grid");
    if (a->first_azimuth_line != 0 || a->first_range_sample != 0)
        return set_err(c, GSLC_EINVAL, "the input raster starts at the radar grid's first line and sample");
    return geocode_slc_impl(c, a, (cudaStream_t)stream, nullptr, nullptr, nullptr, lines_per_block);
}

// ---------------------------------------------------------------------------
// Host radar blocks and DEM window uploaded while the geogrid's row bands
// compute (gslc_geocode_slc_host_io).
namespace {

struct IoBand {
    int64_t row0, rows;
    int64_t az_lo, az_hi;     // radar lines of the blocks (block-relative) the band's chips read
    int64_t dem_lo, dem_hi;   // DEM window rows its splines read
};

// The lines and rows a band of geogrid rows reads, from the pixel centres of
// its perimeter (every eighth of each edge) at the lowest and highest
// heights a DEM can hold (-500 and 9000 m), by the zero-Doppler geo2rdr on
// the host: the sinc chip adds 4 lines on each side, the spline rows -1..+4
// of the point's row.  A band whose points all fail takes everything.  The
// plan only orders the uploads: a chip or spline outside the uploaded rows
// raises error bit 3 and the call repeats its bands.
void plan_io_band(const GeoParams& p, const Orbit& ob, const gslc_geocode_args* a, int64_t margin, IoBand& b) {
    const int64_t inL = a->rdr_length;
    const int64_t demL = p.dem.have_raster ? p.dem.length : 0;
    double az_min = INFINITY, az_max = -INFINITY, r_min = INFINITY, r_max = -INFINITY;
    bool any = false;
    const int64_t W = p.gw;
    for (int e = 0; e < 4; ++e) {
        for (int k = 0; k <= 8; ++k) {
            int64_t line, pix;
            if (e == 0) { line = b.row0; pix = (W - 1) * k / 8; }
            else if (e == 1) { line = b.row0 + b.rows - 1; pix = (W - 1) * k / 8; }
            else if (e == 2) { line = b.row0 + (b.rows - 1) * k / 8; pix = 0; }
            else { line = b.row0 + (b.rows - 1) * k / 8; pix = W - 1; }
            const double x = p.gx0 + p.gdx * ((double)pix + 0.5);
            const double y = p.gy0 + p.gdy * ((double)line + 0.5);
            double lon, lat;
            if (p.geo_is_lonlat) {
                lon = x * PI / 180.0;
                lat = y * PI / 180.0;
            } else if (!utm_inverse(p.utm, x, y, lon, lat)) {
                continue;
            }
            if (demL > 0) {
                double row = NAN;
                if (p.dem.epsg_is_lonlat) {
                    row = ((lat * 180.0) / PI - p.dem.y_start) / p.dem.dy;
                } else {
                    double X, Y;
                    if (utm_forward(p.dem.utm, lon, lat, X, Y)) row = (Y - p.dem.y_start) / p.dem.dy;
                }
                if (std::isfinite(row)) {
                    r_min = std::min(r_min, row);
                    r_max = std::max(r_max, row);
                }
            }
            for (const double h : {-500.0, 9000.0}) {
                const V3 xyz = lonlat_to_xyz(p.ell_a, p.ell_e2, lon, lat, h);
                if (!p.t_mid_in_orbit) continue;
                const V3 rvec = vsub(xyz, p.pos0);
                double t = p.t_mid, R = 0.0;
                const double dt = -vdot(rvec, p.vel0) * p.inv_vv0;
                bool ok = std::fabs(dt) < p.thr;
                if (!ok)
                    ok = ob.legendre ? geo2rdr_zero_doppler_orbit(ob, xyz, p.thr, std::max(p.maxiter, 2), t, dt, R)
                                     : geo2rdr_zero_doppler_seg(ob, ob.seg, xyz, p.thr, std::max(p.maxiter, 2), t, dt, R);
                if (!ok) continue;
                const double azc = (t - p.rg_t0) * p.rg_prf - p.az_first_d;
                az_min = std::min(az_min, azc);
                az_max = std::max(az_max, azc);
                any = true;
            }
        }
    }
    if (any) {
        b.az_lo = std::max<int64_t>(0, (int64_t)std::floor(az_min) - 4 - margin);
        b.az_hi = std::min<int64_t>(inL - 1, (int64_t)std::ceil(az_max) + 4 + margin);
        if (b.az_lo > b.az_hi) b.az_lo = b.az_hi = std::min<int64_t>(std::max<int64_t>(0, b.az_lo), inL - 1);
    } else {
        b.az_lo = 0;
        b.az_hi = inL - 1;
    }
    if (demL > 0 && std::isfinite(r_min)) {
        b.dem_lo = std::max<int64_t>(0, (int64_t)std::floor(r_min) - 1 - margin);
        b.dem_hi = std::min<int64_t>(demL - 1, (int64_t)std::ceil(r_max) + 4 + margin);
        if (b.dem_lo > b.dem_hi) b.dem_lo = b.dem_hi = std::min<int64_t>(std::max<int64_t>(0, b.dem_lo), demL - 1);
    } else {
        b.dem_lo = 0;
        b.dem_hi = std::max<int64_t>(demL - 1, 0);
    }
}

cudaEvent_t io_event(gslc_ctx* c, size_t i) {
    while (c->io_ev.size() <= i) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        c->io_ev.push_back(e);
    }
    return c->io_ev[i];
}

}  // namespace

extern "C" int gslc_geocode_slc_host_io(gslc_ctx* c, const gslc_geocode_args* a, const gslc_host_io* io,
                                        void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    c->io_reruns = 0;
    if (!a || !io || !io->rdr_blocks) return set_err(c, GSLC_EINVAL, "null arguments");
    if (a->inplace_deramp) return set_err(c, GSLC_EINVAL, "in-place deramp needs device radar blocks");
    if (io->dem && io->dem_stride < a->dem.data_width)
        return set_err(c, GSLC_EINVAL, "host DEM row stride shorter than the DEM window");
    cudaStream_t stream = (cudaStream_t)stream_;
    GeoParams p;
    std::vector<double> coef;
    int st = prepare_geocode(c, a, p, coef);
    if (st == GSLC_EMPTY_GRID) return GSLC_OK;
    if (st != GSLC_OK) return st;
    const gslc_radar_grid& rg = a->radar_grid;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    // The upload stream runs at the highest priority: its deramp chunks then
    // take SM slots ahead of the band kernels already resident, so the
    // uploads behind them (and the enqueue loop, which blocks on pageable
    // DEM copies) do not wait for a band to drain (frame: enqueue 30 ->
    // 6 ms of the 36 ms call).
    if (!c->h2d_stream) {
        int lo = 0, hi = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi)) != cudaSuccess) return cuda_err(c, e, "stream priority");
        if ((e = cudaStreamCreateWithPriority(&c->h2d_stream, cudaStreamNonBlocking, hi)) != cudaSuccess) {
            c->h2d_stream = nullptr;
            return cuda_err(c, e, "stream");
        }
    }
    for (cudaStream_t* s : {&c->aux_stream, &c->copy_stream})
        if (!*s && (e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking)) != cudaSuccess) {
            *s = nullptr;
            return cuda_err(c, e, "stream");
        }
    if (coef.size() > c->orbit_cap) {
        if (c->d_orbit) cudaFree(c->d_orbit);
        c->d_orbit = nullptr;
        e = cudaMalloc(&c->d_orbit, coef.size() * sizeof(double));
        if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc orbit");
        c->orbit_cap = coef.size();
    }
    // host copy of the orbit tables for the band plan
    GeoParams ph = p;
    bind_orbit(ph, coef.data());
    e = cudaMemcpyAsync(c->d_orbit, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cuda_err(c, e, "orbit upload");
    bind_orbit(p, c->d_orbit);
    p.sinc = c->d_sinc;
    p.err = c->d_err;
    p.dem.err = c->d_err;
    e = cudaMemsetAsync(c->d_err, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return cuda_err(c, e, "memset");

    const int64_t inL = a->rdr_length, inW = a->rdr_width, nrdr = inL * inW;
    const size_t sbytes = p.rdr_c32 ? 4 : 8;
    const int64_t gl = p.gl, gw = p.gw;
    const bool deramp = !p.carriers_zero && nrdr > 0 && !a->rdr_deramped;
    std::vector<void*> scratch;
    std::vector<const float2*> rdr(a->n_blocks);
    for (int b = 0; b < a->n_blocks; ++b) rdr[b] = (const float2*)a->rdr_blocks[b];
    std::vector<float2*> deramp_dst(a->n_blocks, nullptr);
    auto fail = [&](int code) {
        for (void* s : scratch) cudaFreeAsync(s, stream);
        cudaStreamSynchronize(c->h2d_stream);
        cudaStreamSynchronize(c->aux_stream);
        cudaStreamSynchronize(c->copy_stream);
        return code;
    };
    if (deramp) {
        // complex64 staging is deramped where it lies; complex32 into complex64 scratch
        for (int b = 0; b < a->n_blocks; ++b) {
            if (!p.rdr_c32) {
                deramp_dst[b] = (float2*)a->rdr_blocks[b];
                continue;
            }
            void* buf = nullptr;
            e = cudaMallocAsync(&buf, nrdr * sizeof(float2), stream);
            if (e != cudaSuccess) return fail(cuda_err(c, e, "cudaMallocAsync deramp scratch"));
            scratch.push_back(buf);
            deramp_dst[b] = (float2*)buf;
            rdr[b] = (const float2*)buf;
        }
    }

    // bands, planned and ordered by the first radar line they read
    const int nb_want = io->bands > 0 ? io->bands : 6;
    int64_t band_rows = ((gl + nb_want - 1) / nb_want + 31) / 32 * 32;
    const int nb0 = (int)((gl + band_rows - 1) / band_rows);
    // the first and last row bands are split, an eighth of a band at the
    // geogrid's edge: whichever end the uploads start from, the first
    // kernel waits for fewer radar lines and the last band's copy back is
    // shorter (frame: 38.0 -> 37.7 ms per call).  Every band starts on a
    // multiple of 32 rows, the tile height, so that the tiles (and their
    // UTM fits) are those of one launch over the whole geogrid.
    std::vector<IoBand> bands;
    {
        const int64_t q = std::max<int64_t>(32, (band_rows / 8 + 31) / 32 * 32);
        for (int i = 0; i < nb0; ++i) {
            const int64_t r0 = (int64_t)i * band_rows, rows = std::min(band_rows, gl - r0);
            IoBand x{};
            if ((i == 0 || i == nb0 - 1) && rows > 2 * q) {
                const int64_t cut = i == 0 ? q : (rows - q) / 32 * 32;
                x.row0 = r0; x.rows = cut; bands.push_back(x);
                x.row0 = r0 + cut; x.rows = rows - cut; bands.push_back(x);
            } else {
                x.row0 = r0; x.rows = rows; bands.push_back(x);
            }
        }
        for (IoBand& x : bands) plan_io_band(ph, ph.orbit, a, io->margin, x);
    }
    const int nb = (int)bands.size();
    // by first line, then last: where several bands start at the radar grid's
    // first line (the clamp), the one needing the fewest lines goes first, so
    // the first kernel waits for the shortest upload (frame: the first band's
    // upload 3558 -> 1125 lines, its kernel starting 0.42 instead of 1.24 ms
    // into the call)
    std::stable_sort(bands.begin(), bands.end(), [](const IoBand& x, const IoBand& y) {
        return x.az_lo != y.az_lo ? x.az_lo < y.az_lo : x.az_hi < y.az_hi;
    });

    // uploads on h2d_stream: a band's missing lines (deramped there) and DEM rows, then an event
    const int64_t demL = (io->dem && p.dem.have_raster) ? p.dem.length : 0;
    const int64_t demW = p.dem.have_raster ? p.dem.width : 0;
    int64_t u0 = 0, u1 = -1, d0 = 0, d1 = -1;   // uploaded lines [u0, u1] and DEM rows [d0, d1]
    size_t evn = 0;
    cudaEvent_t ev_start = io_event(c, evn++);
    if (!ev_start) return fail(set_err(c, GSLC_ECUDA, "event"));
    e = cudaEventRecord(ev_start, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->h2d_stream, ev_start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->aux_stream, ev_start, 0);
    if (e != cudaSuccess) return fail(cuda_err(c, e, "stream order"));
    const int32_t src_c32 = p.rdr_c32;
    auto upload_lines = [&](int64_t l0, int64_t l1) -> cudaError_t {   // [l0, l1]
        if (l1 < l0) return cudaSuccess;
        cudaError_t r = cudaSuccess;
        for (int b = 0; b < a->n_blocks && r == cudaSuccess; ++b)
            r = cudaMemcpyAsync((char*)a->rdr_blocks[b] + l0 * inW * sbytes,
                                (const char*)io->rdr_blocks[b] + l0 * inW * sbytes, (size_t)((l1 - l0 + 1) * inW) * sbytes,
                                cudaMemcpyHostToDevice, c->h2d_stream);
        if (r != cudaSuccess || !deramp) return r;
        for (int b = 0; b < a->n_blocks && r == cudaSuccess; ++b) {
            DerampParams dp;
            std::memset(&dp, 0, sizeof(dp));
            dp.src = (const float2*)((const char*)a->rdr_blocks[b] + l0 * inW * sbytes);
            dp.dst = deramp_dst[b] + l0 * inW;
            dp.src_c32 = src_c32;
            dp.inL = l1 - l0 + 1; dp.inW = inW;
            dp.az_first = a->first_azimuth_line + l0; dp.rg_first = a->first_range_sample;
            dp.rg_t0 = rg.sensing_start; dp.rg_prf = rg.prf; dp.rg_r0 = rg.starting_range;
            dp.rg_dr = rg.range_pixel_spacing;
            dp.inv_prf = 1.0 / rg.prf;
            dp.az_car = p.az_car; dp.rg_car = p.rg_car;
            r = launch_deramp(dp, c->h2d_stream, &c->launches);
        }
        return r;
    };
    auto upload_dem = [&](int64_t r0, int64_t r1) -> cudaError_t {
        if (r1 < r0 || demL == 0) return cudaSuccess;
        return cudaMemcpy2DAsync((float*)p.dem.data + r0 * p.dem.stride, p.dem.stride * sizeof(float),
                                 io->dem + r0 * io->dem_stride, io->dem_stride * sizeof(float), demW * sizeof(float),
                                 (size_t)(r1 - r0 + 1), cudaMemcpyHostToDevice, c->h2d_stream);
    };
    if (deramp) p.rdr_c32 = 0;
    const size_t esz = geo_pixel_bytes(a->geo_format);
    std::vector<cudaEvent_t> band_done(nb);
    for (int i = 0; i < nb && e == cudaSuccess; ++i) {
        IoBand& B = bands[i];
        if (u1 < u0) {
            e = upload_lines(B.az_lo, B.az_hi);
            u0 = B.az_lo; u1 = B.az_hi;
        } else {
            if (B.az_lo < u0) { e = upload_lines(B.az_lo, u0 - 1); u0 = B.az_lo; }
            if (e == cudaSuccess && B.az_hi > u1) { e = upload_lines(u1 + 1, B.az_hi); u1 = B.az_hi; }
        }
        if (e == cudaSuccess && demL > 0) {
            if (d1 < d0) {
                e = upload_dem(B.dem_lo, B.dem_hi);
                d0 = B.dem_lo; d1 = B.dem_hi;
            } else {
                if (B.dem_lo < d0) { e = upload_dem(B.dem_lo, d0 - 1); d0 = B.dem_lo; }
                if (e == cudaSuccess && B.dem_hi > d1) { e = upload_dem(d1 + 1, B.dem_hi); d1 = B.dem_hi; }
            }
        }
        cudaEvent_t ready = io_event(c, evn++);
        if (!ready) return fail(set_err(c, GSLC_ECUDA, "event"));
        if (e == cudaSuccess) e = cudaEventRecord(ready, c->h2d_stream);
        cudaStream_t s = (i & 1) ? c->aux_stream : stream;
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ready, 0);
        if (e != cudaSuccess) break;
        // the band's kernel, reading only what has arrived
        GeoParams q = p;
        q.avail_az_lo = u0; q.avail_az_hi = u1;
        if (demL > 0) { q.dem.avail_lo = (int32_t)d0; q.dem.avail_hi = (int32_t)d1; }
        q.geo_row0 = B.row0;
        q.gl = B.rows;
        const int64_t off = B.row0 * gw;
        q.mask = a->mask ? a->mask + off : nullptr;
        q.carrier_out = a->carrier_phase ? a->carrier_phase + off : nullptr;
        q.flatten_out = a->flatten_phase ? a->flatten_phase + off : nullptr;
        q.az_out = a->az_index ? a->az_index + off : nullptr;
        q.rg_out = a->rg_index ? a->rg_index + off : nullptr;
        for (int b0 = 0; b0 < a->n_blocks && e == cudaSuccess; b0 += MAX_BLOCKS) {
            q.nblk = std::min(MAX_BLOCKS, a->n_blocks - b0);
            for (int b = 0; b < q.nblk; ++b) {
                q.rdr[b] = rdr[b0 + b];
                q.geo[b] = (float2*)((char*)a->geo_blocks[b0 + b] + off * esz);
            }
            e = launch_geocode(q, a->geo2rdr_precision, s, &c->launches);
        }
        band_done[i] = io_event(c, evn++);
        if (!band_done[i]) return fail(set_err(c, GSLC_ECUDA, "event"));
        if (e == cudaSuccess) e = cudaEventRecord(band_done[i], s);
    }
    if (e != cudaSuccess) return fail(cuda_err(c, e, "pipelined geocode"));
    // the rest of the radar blocks and DEM window (left complete on the device)
    if (u1 < u0) { e = upload_lines(0, inL - 1); u0 = 0; u1 = inL - 1; }
    if (e == cudaSuccess && u0 > 0) e = upload_lines(0, u0 - 1);
    if (e == cudaSuccess && u1 < inL - 1) e = upload_lines(u1 + 1, inL - 1);
    if (e == cudaSuccess && demL > 0) {
        if (d1 < d0) e = upload_dem(0, demL - 1);
        else {
            if (d0 > 0) e = upload_dem(0, d0 - 1);
            if (e == cudaSuccess && d1 < demL - 1) e = upload_dem(d1 + 1, demL - 1);
        }
    }
    // each band's outputs to the host behind its kernel (queued after every
    // launch: a pageable destination makes the call wait for its copy)
    for (int i = 0; i < nb && e == cudaSuccess && io->geo_blocks; ++i) {
        const IoBand& B = bands[i];
        const int64_t off = B.row0 * gw;
        e = cudaStreamWaitEvent(c->copy_stream, band_done[i], 0);
        for (int b = 0; b < a->n_blocks && e == cudaSuccess; ++b)
            e = cudaMemcpyAsync((char*)io->geo_blocks[b] + off * esz, (const char*)a->geo_blocks[b] + off * esz,
                                (size_t)(B.rows * gw) * esz, cudaMemcpyDeviceToHost, c->copy_stream);
        if (e == cudaSuccess && io->mask && a->mask)
            e = cudaMemcpyAsync(io->mask + off, a->mask + off, (size_t)(B.rows * gw), cudaMemcpyDeviceToHost,
                                c->copy_stream);
    }
    if (e != cudaSuccess) return fail(cuda_err(c, e, "pipelined geocode"));
    cudaEvent_t all_in = io_event(c, evn++), aux_done = io_event(c, evn++), out_done = io_event(c, evn++);
    if (!all_in || !aux_done || !out_done) return fail(set_err(c, GSLC_ECUDA, "event"));
    if (e == cudaSuccess) e = cudaEventRecord(all_in, c->h2d_stream);
    if (e == cudaSuccess) e = cudaEventRecord(aux_done, c->aux_stream);
    if (e == cudaSuccess) e = cudaEventRecord(out_done, c->copy_stream);
    for (cudaEvent_t ev : {all_in, aux_done, out_done})
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ev, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(cuda_err(c, e, "pipelined geocode"));
    if (c->h_err[0] & 8) {
        // a chip or spline read beyond what had arrived: every band again,
        // now that all has (the same values wherever the first pass was right)
        c->io_reruns = 1;
        e = cudaMemsetAsync(c->d_err, 0, sizeof(int32_t), stream);
        for (int i = 0; i < nb && e == cudaSuccess; ++i) {
            const IoBand& B = bands[i];
            GeoParams q = p;
            q.geo_row0 = B.row0;
            q.gl = B.rows;
            const int64_t off = B.row0 * gw;
            q.mask = a->mask ? a->mask + off : nullptr;
            q.carrier_out = a->carrier_phase ? a->carrier_phase + off : nullptr;
            q.flatten_out = a->flatten_phase ? a->flatten_phase + off : nullptr;
            q.az_out = a->az_index ? a->az_index + off : nullptr;
            q.rg_out = a->rg_index ? a->rg_index + off : nullptr;
            for (int b0 = 0; b0 < a->n_blocks && e == cudaSuccess; b0 += MAX_BLOCKS) {
                q.nblk = std::min(MAX_BLOCKS, a->n_blocks - b0);
                for (int b = 0; b < q.nblk; ++b) {
                    q.rdr[b] = rdr[b0 + b];
                    q.geo[b] = (float2*)((char*)a->geo_blocks[b0 + b] + off * esz);
                }
                e = launch_geocode(q, a->geo2rdr_precision, stream, &c->launches);
            }
        }
        if (e == cudaSuccess && io->geo_blocks) {
            for (int b = 0; b < a->n_blocks && e == cudaSuccess; ++b)
                e = cudaMemcpyAsync(io->geo_blocks[b], a->geo_blocks[b], (size_t)(gl * gw) * esz, cudaMemcpyDeviceToHost,
                                    stream);
            if (e == cudaSuccess && io->mask && a->mask)
                e = cudaMemcpyAsync(io->mask, a->mask, (size_t)(gl * gw), cudaMemcpyDeviceToHost, stream);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return fail(cuda_err(c, e, "pipelined geocode re-run"));
    }
    for (void* s : scratch) cudaFreeAsync(s, stream);
    return device_status(c, c->h_err[0]);
}

extern "C" int gslc_last_io_reruns(const gslc_ctx* c) { return c ? c->io_reruns : 0; }

extern "C" int gslc_geocode_slc_to_host(gslc_ctx* c, const gslc_geocode_args* a, void* const* host_geo_blocks,
                                        uint8_t* host_mask, void* stream) {
    if (!c) return GSLC_EINVAL;
    if (!a || !host_geo_blocks) return set_err(c, GSLC_EINVAL, "null arguments");
    const bool empty = (int64_t)a->geo_grid.length * a->geo_grid.width <= 0;   // nothing to copy
    for (int b = 0; b < a->n_blocks && !empty; ++b)
        if (!host_geo_blocks[b]) return set_err(c, GSLC_EINVAL, "null host geo block");
    return geocode_slc_impl(c, a, (cudaStream_t)stream, host_geo_blocks, host_mask);
}

// ---- raster geocoder (cuda/geocode/Geocode.cu:652-864) --------------------
extern "C" int gslc_geocode_rasters(gslc_ctx* c, const gslc_raster_geocode_args* r, void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    if (!r) return set_err(c, GSLC_EINVAL, "null arguments");
    if (r->n_rasters < 0 || (r->n_rasters > 0 && (!r->input_rasters || !r->output_rasters || !r->invalid_values)) ||
        (r->n_rasters == 0 && !r->az_index && !r->rg_index))
        return set_err(c, GSLC_EINVAL, "number of input and output rasters not equal");
    if (r->lines_per_block < 1) return set_err(c, GSLC_EINVAL, "lines_per_block must be positive");
    if (r->maxiter < 0) return set_err(c, GSLC_EINVAL, "maxiter must be non-negative");
    if (!(r->delta_range != 0.0)) return set_err(c, GSLC_EINVAL, "delta_range must be non-zero");
    for (int i = 0; i < r->n_rasters; ++i)
        if (std::fabs(r->invalid_values[i]) > 3.4028234663852886e38)   // Geocode.cu:332-337 (NaN passes)
            return set_err(c, GSLC_EINVAL, "float32-type datatype invalid value exceeds type max");
    cudaStream_t stream = (cudaStream_t)stream_;
    // the shared geometry through the geocodeSlc preparation: no slicing,
    // carriers or flattening
    gslc_geocode_args a;
    std::memset(&a, 0, sizeof(a));
    a.radar_grid = a.sliced_radar_grid = r->radar_grid;
    a.geo_grid = r->geo_grid;
    a.orbit = r->orbit;
    a.native_doppler = r->native_doppler;
    a.image_grid_doppler = r->doppler;
    a.az_time_correction = r->az_time_correction;
    a.srange_correction = r->srange_correction;
    a.az_carrier.kind = a.rg_carrier.kind = 0;      // default LUT2d: zero
    a.ellipsoid_a = r->ellipsoid_a;
    a.ellipsoid_e2 = r->ellipsoid_e2;
    a.threshold_geo2rdr = r->threshold;
    a.numiter_geo2rdr = r->maxiter;
    a.n_blocks = r->n_rasters;
    a.rdr_length = r->radar_grid.length;
    a.rdr_width = r->radar_grid.width;
    a.rdr_blocks = r->input_rasters;
    a.geo_blocks = r->output_rasters;
    // coordinates only: one placeholder block for the argument checks; the
    // launches below run with no rasters
    void* const none[1] = {nullptr};
    if (r->n_rasters == 0) {
        a.n_blocks = 1;
        a.rdr_blocks = none;
        a.geo_blocks = none;
    }
    a.dem = r->dem;
    a.dem_margin = r->dem_margin;
    a.geo2rdr_precision = r->geo2rdr_precision;
    a.subswaths = r->subswaths;
    GeoParams p;
    std::vector<double> coef;
    int st = prepare_geocode(c, &a, p, coef);
    if (st == GSLC_EMPTY_GRID) return GSLC_OK;
    if (st != GSLC_OK) return st;
    p.raster = 1;
    p.dop_dr = r->delta_range;
    p.mask = nullptr;
    p.az_out = r->az_index;
    p.rg_out = r->rg_index;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    if (coef.size() > c->orbit_cap) {
        if (c->d_orbit) cudaFree(c->d_orbit);
        c->d_orbit = nullptr;
        e = cudaMalloc(&c->d_orbit, coef.size() * sizeof(double));
        if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc orbit");
        c->orbit_cap = coef.size();
    }
    e = cudaMemcpyAsync(c->d_orbit, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return cuda_err(c, e, "orbit upload");
    bind_orbit(p, c->d_orbit);
    p.sinc = c->d_sinc;
    p.err = c->d_err;
    e = cudaMemsetAsync(c->d_err, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return cuda_err(c, e, "memset");
    if (c->timing) cudaEventRecord(c->ev[0], stream);
    const gslc_geo_grid& gg = r->geo_grid;
    const int lpb = r->lines_per_block;
    const int n_geo_blocks = (gg.length + lpb - 1) / lpb;
    for (int gb = 0; gb < n_geo_blocks; ++gb) {
        // Geocode.cu:393-418: block extent and its own DEM window
        const int line_start = gb * lpb;
        const int block_length = std::min(lpb, gg.length - line_start);
        gslc_dem_window w;
        st = gslc_compute_dem_window_block(&r->dem, &gg, line_start, block_length, gg.width, r->dem_margin, &w);
        if (st == GSLC_EPROJ) return set_err(c, GSLC_EINVAL, "projection transformation between geogrid and DEM failed");
        if (st != GSLC_OK) return set_err(c, st, "unsupported or invalid DEM raster");
        if (w.wraps) return set_err(c, GSLC_EUNSUPPORTED, "DEM window crossing the DEM file discontinuity");
        if ((st = bind_dem_window(c, r->dem, w, p.dem))) return st;
        p.geo_row0 = line_start;
        p.gl = block_length;
        const int64_t off = (int64_t)line_start * gg.width;
        p.az_out = r->az_index ? r->az_index + off : nullptr;
        p.rg_out = r->rg_index ? r->rg_index + off : nullptr;
        // no rasters: one launch for the radar coordinates alone
        for (int b0 = 0; b0 < std::max(r->n_rasters, 1); b0 += MAX_BLOCKS) {
            p.nblk = std::min(MAX_BLOCKS, r->n_rasters - b0);
            for (int b = 0; b < p.nblk; ++b) {
                p.rdr[b] = (const float2*)r->input_rasters[b0 + b];
                p.geo[b] = (float2*)r->output_rasters[b0 + b] + off;
                const double v = r->invalid_values[b0 + b];
                p.inv_blk[b] = std::isnan(v) ? NAN : (float)v;   // Geocode.cu:700-712
            }
            e = launch_geocode(p, r->geo2rdr_precision, stream, &c->launches);
            if (e != cudaSuccess) return cuda_err(c, e, "geocode launch");
        }
    }
    if (c->timing) cudaEventRecord(c->ev[1], stream);
    e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_err(c, e, "geocode");
    if (c->timing) {
        cudaEventElapsedTime(&c->ms_geocode, c->ev[0], c->ev[1]);
        c->ms_deramp = 0.f;
    }
    return device_status(c, c->h_err[0]);
}

extern "C" int gslc_ctx_set_stage_wait(gslc_ctx* c, int64_t clocks) {
    if (!c) return GSLC_EINVAL;
    c->stage_wait = clocks > 0 ? clocks : 0;
    return GSLC_OK;
}

extern "C" int gslc_ctx_set_timing(gslc_ctx* c, int32_t enable) {
    if (!c) return GSLC_EINVAL;
    cudaSetDevice(c->device);
    if (enable && !c->ev[0]) {
        for (auto& e : c->ev)
            if (cudaEventCreate(&e) != cudaSuccess) return set_err(c, GSLC_ECUDA, "cudaEventCreate");
    }
    c->timing = enable ? 1 : 0;
    return GSLC_OK;
}

extern "C" int gslc_last_kernel_ms(const gslc_ctx* c, float* geocode_ms, float* deramp_ms) {
    if (!c || !c->timing) return GSLC_EINVAL;
    if (geocode_ms) *geocode_ms = c->ms_geocode;
    if (deramp_ms) *deramp_ms = c->ms_deramp;
    return GSLC_OK;
}

extern "C" int gslc_probe_fp64_gflops(gslc_ctx* c, double* gflops) {
    if (!c || !gflops) return GSLC_EINVAL;
    cudaSetDevice(c->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int blocks = sms * 8, iters = 4096;
    double* out = nullptr;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double));
    if (e != cudaSuccess) return cuda_err(c, e, "probe alloc");
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0, 0);
        e = probe_fp64(out, blocks, iters, 0);
        cudaEventRecord(e1, 0);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_err(c, e, "probe launch");
    const double flops = 2.0 * 8.0 * iters * (double)blocks * 256.0;
    *gflops = flops / (best * 1e-3) / 1e9;
    return GSLC_OK;
}

// ---- block planning (geometry/boundingbox.cpp:434-641) --------------------
extern "C" int gslc_radar_bbox_blocks(gslc_ctx* c, const gslc_bbox_args* a, gslc_radar_bbox* out, void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    if (!a || (a->n_blocks > 0 && (!a->blocks || !out))) return set_err(c, GSLC_EINVAL, "null arguments");
    // boundingbox.cpp:444-454
    if (a->max_height < a->min_height) return set_err(c, GSLC_EINVAL, "max_height <  min_height");
    if (a->margin < 0)
        return set_err(c, GSLC_EINVAL,
                       "Margin should be a nonnegative number. " + std::to_string(a->margin) + " requested.");
    if (a->n_blocks < 0 || a->n_blocks > (1 << 24)) return set_err(c, GSLC_EINVAL, "n_blocks out of range");
    // bounds on the work of one thread (the reference has none): a sequence
    // runs at most expansion x maxiter Newton iterations
    if (a->geogrid_expansion_threshold < 0 || a->geogrid_expansion_threshold > 10000 || a->maxiter < 0 ||
        a->maxiter > 1000)
        return set_err(c, GSLC_EINVAL, "geogrid_expansion_threshold must be in [0, 10000] and maxiter in [0, 1000]");
    if (!grid_ok(a->radar_grid)) return set_err(c, GSLC_EINVAL, "invalid radar grid");
    if (!is_lonlat_or_utm(a->epsg)) return set_err(c, GSLC_EUNSUPPORTED, "geogrid EPSG must be 4326 or UTM");
    if (int st = check_orbit(c, a->orbit)) return st;
    if (int st = check_lut(c, a->doppler, "doppler")) return st;
    if (a->n_blocks == 0) return GSLC_OK;
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");

    PlanParams p;
    std::memset(&p, 0, sizeof(p));
    std::vector<double> coef;
    orbit_table_cached(c, a->orbit, coef, p.orbit);
    const gslc_radar_grid& rg = a->radar_grid;
    p.n_blocks = a->n_blocks;
    p.geo_is_lonlat = a->epsg == 4326;
    if (!p.geo_is_lonlat) utm_setup(a->epsg, p.utm);
    p.dop = to_lut(a->doppler, c->d_sinc64);
    p.ell_a = WGS84_A;
    p.ell_e2 = WGS84_E2;
    p.t_mid = 0.5 * (rg.sensing_start + grid_stop(rg));     // RadarGridParameters::sensingMid
    p.t0 = rg.sensing_start;
    p.prf = rg.prf;
    p.r0 = rg.starting_range;
    p.dr = rg.range_pixel_spacing;
    p.wvl = rg.wavelength;
    p.look_side = rg.look_side;
    p.maxiter = a->maxiter;
    p.thr = a->threshold;
    p.delta_range = a->delta_range;
    p.hmin = a->min_height;
    p.hmax = a->max_height;
    p.margin = a->margin;
    p.expansion = a->geogrid_expansion_threshold;
    p.length = rg.length;
    p.width = rg.width;

    // one stream-ordered scratch: orbit table, block list, results
    const size_t n = (size_t)a->n_blocks;
    const size_t orb_b = coef.size() * sizeof(double);
    const size_t blk_off = (orb_b + 255) & ~(size_t)255, blk_b = n * 6 * sizeof(double);
    const size_t out_off = (blk_off + blk_b + 255) & ~(size_t)255, out_b = n * 6 * sizeof(int32_t);
    std::vector<double> blocks(n * 6);
    for (size_t i = 0; i < n; ++i) {
        const gslc_geo_block& b = a->blocks[i];
        double* d = &blocks[i * 6];
        d[0] = b.start_x; d[1] = b.start_y; d[2] = b.spacing_x; d[3] = b.spacing_y;
        d[4] = (double)b.width; d[5] = (double)b.length;
    }
    char* buf = nullptr;
    e = cudaMallocAsync((void**)&buf, out_off + out_b, stream);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMallocAsync planner scratch");
    e = cudaMemcpyAsync(buf, coef.data(), orb_b, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + blk_off, blocks.data(), blk_b, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) {
        const double* d_coef = reinterpret_cast<const double*>(buf);
        p.orbit.coef = d_coef;
        p.orbit.seg_ff = reinterpret_cast<const float2*>(d_coef + orbit_segff_offset(p.orbit.n));
        p.orbit.seg = d_coef + orbit_seg_offset(p.orbit.n);
        p.blocks = reinterpret_cast<const double*>(buf + blk_off);
        p.out = reinterpret_cast<int32_t*>(buf + out_off);
        e = launch_radar_bbox(p, stream, &c->launches);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, buf + out_off, out_b, cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(buf, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_err(c, e, "radar bbox");
    return GSLC_OK;
}

// ---- radar grid metadata cubes (geometry/metadataCubes.cpp:276-489) --------
extern "C" int gslc_make_radar_grid_cubes(gslc_ctx* c, const gslc_cube_args* a, void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    if (!a) return set_err(c, GSLC_EINVAL, "null arguments");
    const gslc_geo_grid& gg = a->geo_grid;
    if (a->n_heights < 0 || (a->n_heights > 0 && !a->heights) || gg.width < 0 || gg.length < 0)
        return set_err(c, GSLC_EINVAL, "invalid cube shape");
    if ((int64_t)a->n_heights * gg.length * gg.width > (int64_t)1 << 34)
        return set_err(c, GSLC_EINVAL, "cube larger than 2^34 points");
    if (a->maxiter < 0 || a->maxiter > 1000) return set_err(c, GSLC_EINVAL, "numiter_geo2rdr must be in [0, 1000]");
    if (!grid_ok(a->radar_grid)) return set_err(c, GSLC_EINVAL, "invalid radar grid");
    if (!is_lonlat_or_utm(gg.epsg)) return set_err(c, GSLC_EUNSUPPORTED, "geogrid EPSG must be 4326 or UTM");
    if (int st = check_orbit(c, a->orbit)) return st;
    if (int st = check_lut(c, a->native_doppler, "native_doppler")) return st;
    if (int st = check_lut(c, a->grid_doppler, "grid_doppler")) return st;
    const int64_t npts = (int64_t)a->n_heights * gg.length * gg.width;
    if (npts == 0) return GSLC_OK;
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");

    CubeParams p;
    std::memset(&p, 0, sizeof(p));
    std::vector<double> coef;
    orbit_table_cached(c, a->orbit, coef, p.orbit);
    const gslc_radar_grid& rg = a->radar_grid;
    p.gx0 = gg.start_x; p.gy0 = gg.start_y; p.gdx = gg.spacing_x; p.gdy = gg.spacing_y;
    p.width = gg.width; p.length = gg.length; p.n_heights = a->n_heights;
    p.geo_is_lonlat = gg.epsg == 4326;
    if (!p.geo_is_lonlat) utm_setup(gg.epsg, p.utm);
    p.grid_dop = to_lut(a->grid_doppler, c->d_sinc64);
    p.nat_dop = to_lut(a->native_doppler, c->d_sinc64);
    p.t_mid = 0.5 * (rg.sensing_start + grid_stop(rg));
    p.mid_range = 0.5 * (rg.starting_range + grid_end(rg));      // RadarGridParameters::midRange
    p.wvl = rg.wavelength;
    p.thr = a->threshold;
    p.delta_range = a->delta_range;
    p.look_side = rg.look_side;
    p.maxiter = a->maxiter;
    p.slant_range = a->slant_range; p.azimuth_time = a->azimuth_time;
    p.incidence = a->incidence_angle; p.los_x = a->los_unit_vector_x; p.los_y = a->los_unit_vector_y;
    p.along_x = a->along_track_unit_vector_x; p.along_y = a->along_track_unit_vector_y;
    p.elevation = a->elevation_angle; p.ground_velocity = a->ground_track_velocity;
    p.want_vectors = (p.incidence || p.los_x || p.los_y || p.along_x || p.along_y || p.elevation ||
                      p.ground_velocity) ? 1 : 0;

    // device scratch: orbit table, heights, chain starts / iterates / statuses
    const size_t orb_b = coef.size() * sizeof(double);
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t h_off = up(orb_b), h_b = (size_t)a->n_heights * sizeof(double);
    const size_t sg_off = up(h_off + h_b), pt_b = (size_t)npts * sizeof(double);
    const size_t sn_off = up(sg_off + pt_b), tg_off = up(sn_off + pt_b), tn_off = up(tg_off + pt_b);
    const size_t st_off = up(tn_off + pt_b), total = st_off + (size_t)npts;
    std::vector<double> start_g((size_t)npts, p.t_mid), start_n((size_t)npts, p.t_mid);
    std::vector<double> tg((size_t)npts), tn((size_t)npts);
    std::vector<uint8_t> stat((size_t)npts), prev_stat;
    char* buf = nullptr;
    e = cudaMallocAsync((void**)&buf, total, stream);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMallocAsync cube scratch");
    e = cudaMemcpyAsync(buf, coef.data(), orb_b, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + h_off, a->heights, h_b, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(int32_t), stream);
    const double* d_coef = reinterpret_cast<const double*>(buf);
    p.orbit.coef = d_coef;
    p.orbit.seg_ff = reinterpret_cast<const float2*>(d_coef + orbit_segff_offset(p.orbit.n));
    p.orbit.seg = d_coef + orbit_seg_offset(p.orbit.n);
    p.heights = reinterpret_cast<const double*>(buf + h_off);
    p.start_grid = reinterpret_cast<const double*>(buf + sg_off);
    p.start_native = reinterpret_cast<const double*>(buf + sn_off);
    p.t_grid = reinterpret_cast<double*>(buf + tg_off);
    p.t_native = reinterpret_cast<double*>(buf + tn_off);
    p.status = reinterpret_cast<uint8_t*>(buf + st_off);
    p.err = c->d_err;
    // The reference chains each height layer through its points in row-major
    // order (metadataCubes.cpp:311-413): a point's grid-Doppler solve starts
    // from the previous point's result, or sensingMid after a failure; its
    // native-Doppler solve from the native state of the last point whose grid
    // solve converged (reset to sensingMid after a native failure).  Each
    // pass solves every point from the starts the previous pass implies; the
    // first k points of a chain are exact after k passes.  Where neighbouring
    // points share an azimuth time the reference's solve can stop at its
    // start, so its returned times depend on the visiting order by up to the
    // threshold; the passes stop once no convergence status changes (at least
    // two, so that every point starts warm as in the reference).
    const int64_t plane = (int64_t)gg.length * gg.width;
    constexpr int MAX_PASSES = 16;
    int passes = 0;
    bool settled = false;
    while (e == cudaSuccess && !settled && passes < MAX_PASSES) {
        e = cudaMemcpyAsync(buf + sg_off, start_g.data(), pt_b, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(buf + sn_off, start_n.data(), pt_b, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = launch_radar_grid_cubes(p, stream, &c->launches);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tg.data(), p.t_grid, pt_b, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tn.data(), p.t_native, pt_b, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(stat.data(), p.status, (size_t)npts, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) break;
        ++passes;
        settled = passes > 1 && stat == prev_stat;
        if (settled) break;
        for (int hc = 0; hc < a->n_heights; ++hc) {
            double sg = p.t_mid, sn = p.t_mid;
            for (int64_t q = 0; q < plane; ++q) {
                const int64_t k = hc * plane + q;
                start_g[k] = sg;
                start_n[k] = sn;
                sg = (stat[k] & 1) ? tg[k] : p.t_mid;
                if ((stat[k] & 1) && p.want_vectors) sn = (stat[k] & 2) ? tn[k] : p.t_mid;
            }
        }
        prev_stat = stat;
    }
    c->cube_passes = passes;
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(buf, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_err(c, e, "radar grid cubes");
    if (c->h_err[0] & 1) return set_err(c, GSLC_EPROJ, "Inverse projection transformation failed");
    return GSLC_OK;
}

extern "C" int gslc_last_cube_passes(const gslc_ctx* c) { return c ? c->cube_passes : -1; }

// ---- raster interpolation (cuda/geocode/Geocode.cu:203-287) ----------------
extern "C" int gslc_interpolate_raster(gslc_ctx* c, const double* az_index, const double* rg_index, int64_t n_px,
                                       const void* raster, int64_t length, int64_t width, void* out,
                                       int32_t gdal_type, int32_t method, double invalid_value, void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    if (n_px < 0 || length < 0 || width < 0 || (n_px > 0 && (!az_index || !rg_index || !out || !raster)))
        return set_err(c, GSLC_EINVAL, "invalid raster interpolation arguments");
    int dtype;
    switch (gdal_type) {        // GDALDataType codes
    case 6: dtype = RASTER_F32; break;
    case 10: dtype = RASTER_C64; break;
    case 7: dtype = RASTER_F64; break;
    case 11: dtype = RASTER_C128; break;
    case 1: dtype = RASTER_U8; break;
    case 2: dtype = RASTER_U16; break;
    case 4: dtype = RASTER_U32; break;
    default: return set_err(c, GSLC_EUNSUPPORTED, "raster data type not supported by the CUDA geocoder");
    }
    if (method < 0 || method > 4) return set_err(c, GSLC_EINVAL, "unknown interpolation method");
    if (dtype >= RASTER_U8 && method != 3)
        return set_err(c, GSLC_EINVAL, "int type of raster can only use nearest neighbor interp");
    if (n_px == 0) return GSLC_OK;
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    RasterInterpParams p{};
    p.az = az_index; p.rg = rg_index; p.n = n_px;
    p.rdr = raster; p.L = length; p.W = width;
    p.out = out; p.dtype = dtype; p.method = method; p.invalid = invalid_value;
    p.sinc = c->d_sinc;
    if (method == 0 && (dtype == RASTER_F64 || dtype == RASTER_C128)) {
        if (int st = ensure_sinc64(c)) return st;
        p.sinc = c->d_sinc64;
    }
    e = launch_raster_interp(p, stream, &c->launches);
    if (e != cudaSuccess) return cuda_err(c, e, "raster interpolation");
    return GSLC_OK;
}

extern "C" int gslc_dem_stats(gslc_ctx* c, const float* data, int64_t length, int64_t width, int64_t row_stride,
                              float* mn, float* mx, double* mean, int64_t* n_valid, void* stream_) {
    if (!c) return GSLC_EINVAL;
    c->err.clear();
    c->launches = 0;
    if (!mn || !mx || !mean || !n_valid || length < 0 || width < 0 || (length * width > 0 && !data) ||
        (length > 1 && row_stride < width))
        return set_err(c, GSLC_EINVAL, "invalid DEM raster arguments");
    if (length * width == 0) {
        *mn = std::numeric_limits<float>::max();
        *mx = -std::numeric_limits<float>::max();
        *mean = std::nan("");
        *n_valid = 0;
        return GSLC_OK;
    }
    cudaStream_t stream = (cudaStream_t)stream_;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    void* scratch = nullptr;
    e = cudaMallocAsync(&scratch, dem_stats_scratch_bytes(), stream);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMallocAsync DEM stats scratch");
    DemStats* h = nullptr;
    e = cudaMallocHost((void**)&h, sizeof(DemStats));
    if (e != cudaSuccess) {
        cudaFreeAsync(scratch, stream);
        return cuda_err(c, e, "cudaMallocHost");
    }
    e = launch_dem_stats(data, length, width, row_stride, scratch, h, stream, &c->launches);
    cudaFreeAsync(scratch, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaFreeHost(h);
        return cuda_err(c, e, "DEM stats");
    }
    const long long nv = (long long)(length * width) - h->nan;
    *mn = h->mn;
    *mx = h->mx;
    *mean = h->sum / (double)nv;     // 0 / 0 -> NaN as the reference
    *n_valid = nv;
    cudaFreeHost(h);
    return GSLC_OK;
}

#include <atomic>
#include <mutex>

// ===========================================================================
// Allocation-free entry point.
//
// For callers that must not allocate device memory while they run: serving
// or real-time loops that reserve all of HBM up front under a fixed budget
// (a cudaMalloc there can fail, or stall the device to synchronise), hosts
// whose memory policy forbids allocation after start-up, and frameworks that
// own the device memory pool and hand the geocoder only their own buffers.
// gslc_geocode_slc needs a context, and its constructor and the carrier
// deramp allocate; this variant runs the same kernels with all of its
// scratch in the file-scope device arrays below, held by every GPU that
// loads the library until the process exits (about 33.1 MiB in total).
// ===========================================================================
namespace {

constexpr int64_t NOALLOC_MAX_DERAMP = int64_t(1) << 22;   // complex samples (32 MiB)
constexpr int NOALLOC_MAX_STATE_VECTORS = 256;
constexpr int NOALLOC_MAX_DEVICES = 64;

// deramped radar samples, all blocks back to back
static __device__ __align__(256) float2 g_noalloc_deramp[NOALLOC_MAX_DERAMP];
// sinc kernel table, SINC_SUB x SINC_LEN, in float (the SLC interpolation)
// and in double (LUT2d tables with the sinc method)
static __device__ __align__(256) float g_noalloc_sinc[SINC_SUB * SINC_LEN];
static __device__ __align__(256) double g_noalloc_sinc64[SINC_SUB * SINC_LEN];
// orbit polynomial pieces
static __device__ __align__(256) double g_noalloc_orbit[orbit_table_doubles(NOALLOC_MAX_STATE_VECTORS)];
// error word (bit 0: projection inverse failed); cleared at every call
static __device__ __align__(256) int32_t g_noalloc_err[4];

struct NoallocDevice {
    std::atomic<bool> ready{false};   // set (release) once the fields below hold
    float2* deramp = nullptr;
    float* sinc = nullptr;
    double* sinc64 = nullptr;
    double* orbit = nullptr;
    int32_t* err = nullptr;
};
NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mutex;

int noalloc_fail(char* buf, size_t len, int code, const char* msg) {
    if (buf && len > 0) {
        std::strncpy(buf, msg, len - 1);
        buf[len - 1] = '\0';
    }
    return code;
}

// Once per device, with that device current: the device addresses of the
// static arrays (the host-side names are not device addresses) and the sinc
// table upload, synchronously.
int noalloc_setup(int dev, NoallocDevice& d, char* buf, size_t len) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (d.ready.load(std::memory_order_acquire)) return GSLC_OK;
    cudaError_t e = cudaGetSymbolAddress((void**)&d.deramp, g_noalloc_deramp);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.sinc, g_noalloc_sinc);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.sinc64, g_noalloc_sinc64);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.orbit, g_noalloc_orbit);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&d.err, g_noalloc_err);
    if (e != cudaSuccess) return noalloc_fail(buf, len, GSLC_ECUDA, cudaGetErrorString(e));
    const std::vector<float> table = make_sinc_table();
    const std::vector<double> table64 = make_sinc_table_double();
    e = cudaMemcpy(d.sinc, table.data(), table.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d.sinc64, table64.data(), table64.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return noalloc_fail(buf, len, GSLC_ECUDA, cudaGetErrorString(e));
    d.ready.store(true, std::memory_order_release);
    (void)dev;
    return GSLC_OK;
}

}  // namespace

extern "C" int gslc_geocode_slc_noalloc(const gslc_geocode_args* a, void* stream, char* errbuf, size_t errbuf_len) {
    if (errbuf && errbuf_len) errbuf[0] = '\0';
    if (!a) return noalloc_fail(errbuf, errbuf_len, GSLC_EINVAL, "null arguments");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(errbuf, errbuf_len, GSLC_ECUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return noalloc_fail(errbuf, errbuf_len, GSLC_EUNSUPPORTED, "device index beyond 64");
    NoallocDevice& d = g_noalloc_dev[dev];
    if (!d.ready.load(std::memory_order_acquire)) {
        if (int st = noalloc_setup(dev, d, errbuf, errbuf_len)) return st;
    }
    if (a->orbit.n > NOALLOC_MAX_STATE_VECTORS)
        return noalloc_fail(errbuf, errbuf_len, GSLC_EINVAL,
                            "orbit has more than 256 state vectors (allocation-free limit)");
    if (a->n_blocks < 1 || !a->rdr_blocks || !a->geo_blocks)
        return noalloc_fail(errbuf, errbuf_len, GSLC_EINVAL, "number of geoDataBlocks != number of rdrDataBlocks");

    // A context whose buffers are the static arrays: the regular path then
    // has nothing to allocate (orbit capacity suffices, deramp is in place).
    gslc_ctx c;
    c.device = dev;
    c.no_alloc = true;
    c.d_sinc = d.sinc;
    c.d_sinc64 = d.sinc64;
    c.d_err = d.err;
    static thread_local int32_t h_err[4];
    c.h_err = h_err;
    c.d_orbit = d.orbit;
    c.orbit_cap = orbit_table_doubles(NOALLOC_MAX_STATE_VECTORS);

    AzRg az{}, rg{};
    bool carriers = false;
    if (!to_azrg(&c, a->az_carrier, az, "az_carrier") && !to_azrg(&c, a->rg_carrier, rg, "rg_carrier"))
        carriers = !(az.is_zero && rg.is_zero);
    const int64_t nrdr = a->rdr_length * a->rdr_width;
    // the deramp reads the caller's blocks (complex64 or complex32) and
    // writes the complex64 copies into the static scratch
    if (carriers && !a->inplace_deramp && !a->rdr_deramped && nrdr > 0 && nrdr * a->n_blocks > NOALLOC_MAX_DERAMP)
        return noalloc_fail(errbuf, errbuf_len, GSLC_EINVAL,
                            "radar blocks exceed the allocation-free deramp scratch (4194304 complex samples)");
    const int st = geocode_slc_impl(&c, a, (cudaStream_t)stream, nullptr, nullptr, d.deramp);
    c.d_sinc = nullptr;   // the static arrays are not the context's to free
    c.d_sinc64 = nullptr;
    c.d_err = nullptr;
    c.d_orbit = nullptr;
    c.h_err = nullptr;
    if (st != GSLC_OK) return noalloc_fail(errbuf, errbuf_len, st, c.err.c_str());
    return GSLC_OK;
}

// ===========================================================================
// Batched form: many geocode requests (bursts, tiles of uneven size) in one
// persistent launch over a device tile counter, optionally captured with
// their deramp passes in a CUDA graph and replayed.
// ===========================================================================
struct gslc_batch {
    gslc_ctx* ctx = nullptr;
    int device = 0;
    bool lonlat = false, ff = false;
    int blocks = 0;
    BatchQueue q{};
    GeoParams* d_items = nullptr;
    long long* d_tile_start = nullptr;
    long long* d_counter = nullptr;
    int32_t* d_item_request = nullptr;
    long long* d_request_tiles = nullptr;
    unsigned long long* d_request_done = nullptr;
    int32_t n_requests = 0;
    uint32_t* h_flags = nullptr;        // per-request completion words (mapped host memory) or null
    std::vector<int32_t> no_tiles;      // requests without tiles: flagged by the host at each launch
    double* d_orbit = nullptr;
    float2* d_scratch = nullptr;
    int32_t* d_err = nullptr;
    int32_t h_err[4] = {0, 0, 0, 0};
    cudaStream_t stream = nullptr;  // creation stream: allocation and release order
    std::vector<DerampParams> deramps;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture_stream = nullptr;
    int64_t launches_per_run = 0;
    long long n_tiles = 0;
    // per-request mode: the launch parameters of each entry (its request
    // owner[j]), run as the plain call's kernel on concurrent branch streams
    bool per_request = false;
    std::vector<GeoParams> params;
    std::vector<int> owner;
    std::vector<cudaStream_t> branches;
    cudaEvent_t fork_ev = nullptr;
    std::vector<cudaEvent_t> join_ev;
    unsigned int* d_flags = nullptr;    // device view of h_flags
    std::string err;
};

namespace {

void flag_empty_requests(gslc_batch* b) {
    if (b->h_flags)
        for (int32_t i : b->no_tiles) b->h_flags[i] = 1;
}

int batch_fail(gslc_batch* b, gslc_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    if (b) b->err = m;
    return code;
}

// Per-request mode: after the deramps, each entry's plain kernel on one of
// the branch streams (forked from s and joined back into it), the request's
// completion word behind its last entry.  Concurrent kernels fill each
// other's last waves; inside a graph capture the branches become parallel
// graph paths.
cudaError_t batch_enqueue_per_request(gslc_batch* b, cudaStream_t s) {
    if (b->branches.empty()) {
        // one entry: its kernel and word on the launch stream itself
        cudaError_t e = launch_geocode(b->params[0], b->ff ? 1 : 0, s, nullptr);
        if (e == cudaSuccess && b->d_flags) e = launch_set_flag(b->d_flags + b->owner[0], s, nullptr);
        return e;
    }
    cudaError_t e = cudaEventRecord(b->fork_ev, s);
    for (cudaStream_t br : b->branches)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(br, b->fork_ev, 0);
    const size_t nb = b->branches.size();
    for (size_t j = 0; j < b->params.size() && e == cudaSuccess; ++j) {
        cudaStream_t br = b->branches[j % nb];
        e = launch_geocode(b->params[j], b->ff ? 1 : 0, br, nullptr);
        const bool last = j + 1 == b->params.size() || b->owner[j + 1] != b->owner[j];
        // a request's entries share a branch only when it has one entry; with
        // several, the word waits for all of them on the join below
        if (e == cudaSuccess && b->d_flags && last && (j == 0 || b->owner[j - 1] != b->owner[j]))
            e = launch_set_flag(b->d_flags + b->owner[j], br, nullptr);
    }
    for (size_t k = 0; k < nb && e == cudaSuccess; ++k) {
        e = cudaEventRecord(b->join_ev[k], b->branches[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join_ev[k], 0);
    }
    // requests split over several entries (more than MAX_BLOCKS radar blocks)
    for (size_t j = 0; j < b->params.size() && e == cudaSuccess && b->d_flags; ++j) {
        const bool first = j == 0 || b->owner[j - 1] != b->owner[j];
        const bool last = j + 1 == b->params.size() || b->owner[j + 1] != b->owner[j];
        if (last && !first) e = launch_set_flag(b->d_flags + b->owner[j], s, nullptr);
    }
    return e;
}

cudaError_t batch_enqueue(gslc_batch* b, cudaStream_t s) {
    if (b->per_request) {
        cudaError_t e = cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), s);
        for (const DerampParams& dp : b->deramps) {
            if (e != cudaSuccess) break;
            e = launch_deramp(dp, s, nullptr);
        }
        return e == cudaSuccess ? batch_enqueue_per_request(b, s) : e;
    }
    cudaError_t e = cudaMemsetAsync(b->d_err, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_counter, 0, sizeof(long long), s);
    if (e == cudaSuccess && b->q.done_flags)
        e = cudaMemsetAsync(b->d_request_done, 0, sizeof(unsigned long long) * b->n_requests, s);
    for (const DerampParams& dp : b->deramps) {
        if (e != cudaSuccess) break;
        e = launch_deramp(dp, s, nullptr);
    }
    if (e == cudaSuccess) e = launch_geocode_persistent(b->q, b->lonlat, b->ff, b->blocks, s, nullptr);
    return e;
}

}  // namespace

extern "C" int gslc_batch_create(gslc_ctx* c, const gslc_geocode_args* items, int32_t n, int32_t precision,
                                 const gslc_batch_tuning* tuning, void* stream_, gslc_batch** out) {
    return gslc_batch_create_signaled(c, items, n, precision, tuning, stream_, nullptr, out);
}

extern "C" int gslc_batch_create_signaled(gslc_ctx* c, const gslc_geocode_args* items, int32_t n, int32_t precision,
                                          const gslc_batch_tuning* tuning, void* stream_, uint32_t* done_flags,
                                          gslc_batch** out) {
    if (!c || !out) return GSLC_EINVAL;
    *out = nullptr;
    c->err.clear();
    if (!items || n < 1) return set_err(c, GSLC_EINVAL, "empty batch");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    gslc_batch* b = new (std::nothrow) gslc_batch();
    if (!b) return set_err(c, GSLC_ECUDA, "out of host memory");
    b->ctx = c;
    b->device = c->device;
    b->stream = (cudaStream_t)stream_;
    const cudaStream_t st_ = b->stream;

    const int rpt = tuning ? tuning->rows_per_thread : 0;
    const int ppt = (rpt == 1 || rpt == 2 || rpt == 4) ? rpt : 4;
    std::vector<GeoParams> params;
    std::vector<std::vector<double>> coefs;
    std::vector<int> owner;                 // item index of each params entry
    size_t coef_total = 0, scratch_total = 0;
    bool any_ll = false, any_utm = false;
    for (int i = 0; i < n; ++i) {
        GeoParams p;
        std::vector<double> coef;
        const int st = prepare_geocode(c, &items[i], p, coef);
        if (st == GSLC_EMPTY_GRID) continue;
        if (st != GSLC_OK) {
            gslc_batch_destroy(b);
            return st;
        }
        (p.geo_is_lonlat ? any_ll : any_utm) = true;
        const gslc_geocode_args& a = items[i];
        const int64_t nrdr = a.rdr_length * a.rdr_width;
        if (!p.carriers_zero && nrdr > 0 && !a.inplace_deramp && !a.rdr_deramped)
            scratch_total += (size_t)nrdr * a.n_blocks;
        for (int b0 = 0; b0 < a.n_blocks; b0 += MAX_BLOCKS) {
            GeoParams q = p;
            q.nblk = std::min(MAX_BLOCKS, a.n_blocks - b0);
            params.push_back(q);
            owner.push_back(i);
        }
        coef_total += coef.size();
        coefs.push_back(std::move(coef));
    }
    if (any_ll && any_utm) {
        gslc_batch_destroy(b);
        return set_err(c, GSLC_EUNSUPPORTED, "a batch mixes EPSG:4326 and UTM geogrids");
    }
    b->lonlat = any_ll;
    // float-float only where every request qualifies (one kernel variant per batch)
    b->ff = precision == 1;
    for (const GeoParams& q : params) b->ff = b->ff && ff_eligible(q);
    b->n_requests = n;
    b->h_flags = done_flags;
    {
        std::vector<char> has(n, 0);
        for (int i : owner) has[i] = 1;
        for (int i = 0; i < n; ++i)
            if (!has[i]) b->no_tiles.push_back(i);
    }
    if (params.empty()) {
        flag_empty_requests(b);
        *out = b;
        return GSLC_OK;
    }
    e = cudaMallocAsync((void**)&b->d_orbit, coef_total * sizeof(double), st_);
    if (e == cudaSuccess && scratch_total)
        e = cudaMallocAsync((void**)&b->d_scratch, scratch_total * sizeof(float2), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_items, params.size() * sizeof(GeoParams), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_tile_start, (params.size() + 1) * sizeof(long long), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_counter, sizeof(long long), st_);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_err, sizeof(int32_t) * 4, st_);
    if (e == cudaSuccess && done_flags) {
        e = cudaMallocAsync((void**)&b->d_item_request, params.size() * sizeof(int32_t), st_);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_request_tiles, n * sizeof(long long), st_);
        if (e == cudaSuccess) e = cudaMallocAsync((void**)&b->d_request_done, n * sizeof(unsigned long long), st_);
    }
    if (e != cudaSuccess) {
        gslc_batch_destroy(b);
        return cuda_err(c, e, "batch allocation");
    }
    // orbit polynomials of each item, then bind every params entry
    std::vector<size_t> coef_off;
    size_t off = 0;
    for (const auto& cf : coefs) {
        coef_off.push_back(off);
        // pageable sources are staged by the runtime before the call returns
        e = cudaMemcpyAsync(b->d_orbit + off, cf.data(), cf.size() * sizeof(double), cudaMemcpyHostToDevice, st_);
        if (e != cudaSuccess) break;
        off += cf.size();
    }
    // item index -> coefs index (items with empty grids have no coef)
    std::vector<int> coef_of_item(n, -1);
    {
        int k = 0;
        for (int i = 0, j = 0; i < n && j < (int)owner.size(); ++i)
            if (owner[j] == i) {
                coef_of_item[i] = k++;
                while (j < (int)owner.size() && owner[j] == i) ++j;
            }
    }
    size_t scratch_off = 0;
    std::vector<long long> tile_start(params.size() + 1, 0);
    int last_item = -1, block_base = 0;
    for (size_t j = 0; j < params.size(); ++j) {
        GeoParams& p = params[j];
        const int i = owner[j];
        const gslc_geocode_args& a = items[i];
        block_base = (i == last_item) ? block_base + MAX_BLOCKS : 0;
        last_item = i;
        bind_orbit(p, b->d_orbit + coef_off[coef_of_item[i]]);
        p.sinc = c->d_sinc;
        p.err = b->d_err;
        const int64_t nrdr = a.rdr_length * a.rdr_width;
        for (int k = 0; k < p.nblk; ++k) {
            const float2* src = (const float2*)a.rdr_blocks[block_base + k];
            const float2* use = src;
            if (!p.carriers_zero && nrdr > 0 && !a.rdr_deramped) {
                float2* dst = a.inplace_deramp ? const_cast<float2*>(src) : b->d_scratch + scratch_off;
                if (!a.inplace_deramp) scratch_off += nrdr;
                DerampParams dp;
                std::memset(&dp, 0, sizeof(dp));
                dp.src = src; dp.dst = dst;
                dp.src_c32 = params[j].rdr_c32;
                dp.inL = a.rdr_length; dp.inW = a.rdr_width;
                dp.az_first = a.first_azimuth_line; dp.rg_first = a.first_range_sample;
                const gslc_radar_grid& rg = a.radar_grid;
                dp.rg_t0 = rg.sensing_start; dp.rg_prf = rg.prf; dp.rg_r0 = rg.starting_range;
                dp.rg_dr = rg.range_pixel_spacing; dp.inv_prf = 1.0 / rg.prf;
                dp.az_car = p.az_car; dp.rg_car = p.rg_car;
                b->deramps.push_back(dp);
                use = dst;
            }
            p.rdr[k] = use;
            p.geo[k] = (float2*)a.geo_blocks[block_base + k];
        }
        if (!p.carriers_zero && nrdr > 0 && !a.rdr_deramped) p.rdr_c32 = 0;   // deramped copies are complex64
        const long long tiles = (long long)((p.gw + TILE_X - 1) / TILE_X) * ((p.gl + TILE_Y * ppt - 1) / (TILE_Y * ppt));
        tile_start[j + 1] = tile_start[j] + tiles;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_items, params.data(), params.size() * sizeof(GeoParams), cudaMemcpyHostToDevice,
                            st_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_tile_start, tile_start.data(), tile_start.size() * sizeof(long long),
                            cudaMemcpyHostToDevice, st_);
    if (e != cudaSuccess) {
        gslc_batch_destroy(b);
        return cuda_err(c, e, "batch upload");
    }
    if (e == cudaSuccess && done_flags) {
        std::vector<long long> req_tiles(n, 0);
        for (size_t j = 0; j < params.size(); ++j) req_tiles[owner[j]] += tile_start[j + 1] - tile_start[j];
        e = cudaMemcpyAsync(b->d_item_request, owner.data(), owner.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                            st_);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->d_request_tiles, req_tiles.data(), n * sizeof(long long), cudaMemcpyHostToDevice,
                                st_);
        if (e != cudaSuccess) {
            gslc_batch_destroy(b);
            return cuda_err(c, e, "batch upload");
        }
        unsigned int* dflags = nullptr;
        e = cudaHostGetDevicePointer((void**)&dflags, done_flags, 0);
        if (e != cudaSuccess) {
            gslc_batch_destroy(b);
            return cuda_err(c, e, "done flags are not mapped host memory");
        }
        b->q.item_request = b->d_item_request;
        b->q.request_tiles = b->d_request_tiles;
        b->q.request_done = b->d_request_done;
        b->q.done_flags = dflags;
        b->d_flags = dflags;
    }
    b->n_tiles = tile_start.back();
    b->q.items = b->d_items;
    b->q.tile_start = b->d_tile_start;
    b->q.n_items = (int32_t)params.size();
    b->q.n_tiles = b->n_tiles;
    b->q.counter = b->d_counter;
    b->q.tiles_per_pop = (tuning && tuning->tiles_per_pop > 0) ? tuning->tiles_per_pop : 2;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    b->q.ppt = ppt;
    const int occ = std::max(1, persistent_blocks_per_sm(b->lonlat, b->ff, ppt));
    const int per_sm = (tuning && tuning->blocks_per_sm > 0) ? std::min(tuning->blocks_per_sm, occ) : occ;
    b->blocks = sms * per_sm;
    b->launches_per_run = (int64_t)b->deramps.size() + 1;
    if (tuning && tuning->per_request) {
        if (ppt != 4) {
            gslc_batch_destroy(b);
            return set_err(c, GSLC_EINVAL, "per-request batches use the plain kernel's 32 x 32 tiles (rows_per_thread 4)");
        }
        b->per_request = true;
        b->params = params;
        b->owner = owner;
        // branch streams for two or more entries (one entry runs on the launch stream)
        const int nbr = params.size() > 1 ? (int)std::min<size_t>(4, params.size()) : 0;
        if (nbr > 0) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
        for (int k = 0; k < nbr && e == cudaSuccess; ++k) {
            cudaStream_t br = nullptr;
            cudaEvent_t ev = nullptr;
            e = cudaStreamCreateWithFlags(&br, cudaStreamNonBlocking);
            if (e == cudaSuccess) b->branches.push_back(br);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e == cudaSuccess) b->join_ev.push_back(ev);
        }
        if (e != cudaSuccess) {
            gslc_batch_destroy(b);
            return cuda_err(c, e, "batch streams");
        }
        int64_t flags = 0;
        if (b->d_flags)
            for (size_t j = 0; j < params.size(); ++j)
                if (j + 1 == params.size() || owner[j + 1] != owner[j]) ++flags;
        b->launches_per_run = (int64_t)b->deramps.size() + (int64_t)params.size() + flags;
    }
    if (!tuning || tuning->use_graph) {
        e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = batch_enqueue(b, b->capture_stream);
            e = cudaStreamEndCapture(b->capture_stream, &b->graph);
            if (e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) {
            gslc_batch_destroy(b);
            return cuda_err(c, e, "batch graph capture");
        }
    }
    *out = b;
    return GSLC_OK;
}

extern "C" int gslc_batch_launch(gslc_batch* b, void* stream) {
    if (!b) return GSLC_EINVAL;
    flag_empty_requests(b);
    if (!b->q.n_items) return GSLC_OK;
    cudaError_t e = cudaSetDevice(b->device);
    if (e == cudaSuccess) e = b->exec ? cudaGraphLaunch(b->exec, (cudaStream_t)stream) : batch_enqueue(b, (cudaStream_t)stream);
    if (e != cudaSuccess) return batch_fail(b, b->ctx, GSLC_ECUDA, std::string("batch launch: ") + cudaGetErrorString(e));
    if (b->ctx) b->ctx->launches = b->launches_per_run;
    return GSLC_OK;
}

extern "C" int gslc_batch_status(gslc_batch* b, void* stream) {
    if (!b) return GSLC_EINVAL;
    if (!b->q.n_items) return GSLC_OK;
    cudaError_t e = cudaMemcpyAsync(b->h_err, b->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    // (a pageable destination: the copy has completed when the call returns)
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return batch_fail(b, b->ctx, GSLC_ECUDA, std::string("batch: ") + cudaGetErrorString(e));
    gslc_ctx probe;
    if (const int st = device_status(&probe, b->h_err[0])) return batch_fail(b, b->ctx, st, probe.err);
    return GSLC_OK;
}

extern "C" int gslc_batch_info(const gslc_batch* b, int64_t* n_tiles, int32_t* blocks, int32_t* tiles_per_pop,
                               int64_t* launches) {
    if (!b) return GSLC_EINVAL;
    if (n_tiles) *n_tiles = b->n_tiles;
    if (blocks) *blocks = b->blocks;
    if (tiles_per_pop) *tiles_per_pop = b->q.tiles_per_pop;
    if (launches) *launches = b->launches_per_run;
    return GSLC_OK;
}

extern "C" int gslc_batch_destroy(gslc_batch* b) {
    if (!b) return GSLC_OK;
    cudaSetDevice(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    for (cudaStream_t br : b->branches) cudaStreamDestroy(br);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    for (cudaEvent_t ev : b->join_ev) cudaEventDestroy(ev);
    for (void* ptr : {(void*)b->d_items, (void*)b->d_tile_start, (void*)b->d_counter, (void*)b->d_orbit,
                      (void*)b->d_scratch, (void*)b->d_err, (void*)b->d_item_request, (void*)b->d_request_tiles,
                      (void*)b->d_request_done})
        if (ptr) cudaFreeAsync(ptr, b->stream);
    delete b;
    return GSLC_OK;
}

// ---- GSLC sample codecs (isce3/core/types.py:38-165) ------------------------
namespace {
int codec_call(gslc_ctx* c, int op, const void* src, void* dst, int64_t n, int bits, int word_bytes, void* stream) {
    c->err.clear();
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    c->launches = 0;
    e = launch_codec(op, src, dst, n, bits, word_bytes, (cudaStream_t)stream, &c->launches);
    return e == cudaSuccess ? GSLC_OK : cuda_err(c, e, "codec launch");
}
bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }
}  // namespace

extern "C" int gslc_complex64_to_complex32(gslc_ctx* c, const void* src, void* dst, int64_t n, void* stream) {
    if (!c) return GSLC_EINVAL;
    if (n < 0 || (n > 0 && (!src || !dst || !aligned(src, 8) || !aligned(dst, 4))))
        return set_err(c, GSLC_EINVAL, "complex64 -> complex32: invalid arrays");
    return codec_call(c, 0, src, dst, n, 0, 0, stream);
}

extern "C" int gslc_complex32_to_complex64(gslc_ctx* c, const void* src, void* dst, int64_t n, void* stream) {
    if (!c) return GSLC_EINVAL;
    if (n < 0 || (n > 0 && (!src || !dst || !aligned(src, 4) || !aligned(dst, 8))))
        return set_err(c, GSLC_EINVAL, "complex32 -> complex64: invalid arrays");
    return codec_call(c, 1, src, dst, n, 0, 0, stream);
}

extern "C" int gslc_truncate_mantissa(gslc_ctx* c, void* data, int64_t n_words, int32_t word_bytes,
                                      int32_t significant_bits, void* stream) {
    if (!c) return GSLC_EINVAL;
    if (word_bytes != 2 && word_bytes != 4 && word_bytes != 8)
        return set_err(c, GSLC_EINVAL, "argument z is not complex float or float type");
    const int mant = word_bytes == 2 ? 10 : word_bytes == 4 ? 23 : 52;
    if (!(significant_bits > 0 && significant_bits <= mant))
        return set_err(c, GSLC_EINVAL, "Require 0 < significant_bits <= " + std::to_string(mant));
    if (n_words < 0 || (n_words > 0 && (!data || !aligned(data, (size_t)word_bytes))))
        return set_err(c, GSLC_EINVAL, "truncate_mantissa: invalid array");
    if (significant_bits == mant) return GSLC_OK;
    return codec_call(c, 2, nullptr, data, n_words, significant_bits, word_bytes, stream);
}

// geocodeSlc.cpp:240-274 (carrierPhaseDeramp) as a call of its own: dst =
// src * exp(-i float(rg_carrier + az_carrier)) for a block whose first sample
// is (first_line, first_sample) of radar_grid.  src == dst deramps in place.
extern "C" int gslc_deramp_block(gslc_ctx* c, const gslc_radar_grid* rg, const gslc_azrg_func* az_carrier,
                                 const gslc_azrg_func* rg_carrier, int64_t first_line, int64_t first_sample,
                                 const void* src, void* dst, int64_t length, int64_t width, void* stream) {
    if (!c || !rg || !az_carrier || !rg_carrier || !src || !dst || length < 0 || width < 0) return GSLC_EINVAL;
    c->err.clear();
    DerampParams dp;
    std::memset(&dp, 0, sizeof(dp));
    if (int st = to_azrg(c, *az_carrier, dp.az_car, "az_carrier")) return st;
    if (int st = to_azrg(c, *rg_carrier, dp.rg_car, "rg_carrier")) return st;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaSetDevice");
    dp.src = (const float2*)src;
    dp.dst = (float2*)dst;
    dp.inL = length; dp.inW = width;
    dp.az_first = first_line; dp.rg_first = first_sample;
    dp.rg_t0 = rg->sensing_start; dp.rg_prf = rg->prf; dp.rg_r0 = rg->starting_range;
    dp.rg_dr = rg->range_pixel_spacing; dp.inv_prf = 1.0 / rg->prf;
    if (dp.az_car.is_zero && dp.rg_car.is_zero) {
        if (src != dst) e = cudaMemcpyAsync(dst, src, length * width * sizeof(float2), cudaMemcpyDeviceToDevice,
                                            (cudaStream_t)stream);
        return e == cudaSuccess ? GSLC_OK : cuda_err(c, e, "copy");
    }
    c->launches = 0;
    e = launch_deramp(dp, (cudaStream_t)stream, &c->launches);
    return e == cudaSuccess ? GSLC_OK : cuda_err(c, e, "deramp launch");
}

extern "C" int gslc_host_flags_create(int32_t n, uint32_t** host) {
    if (!host || n < 1) return GSLC_EINVAL;
    cudaError_t e = cudaHostAlloc((void**)host, sizeof(uint32_t) * n, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) return GSLC_ECUDA;
    std::memset(*host, 0, sizeof(uint32_t) * n);
    return GSLC_OK;
}

extern "C" int gslc_host_flags_destroy(uint32_t* host) {
    if (host) cudaFreeHost(host);
    return GSLC_OK;
}
