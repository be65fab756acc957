// Fused SLC geocoding kernel (sm_103a) and the carrier deramp pre-pass.
//
// One thread per output geogrid pixel:
//   map x/y -> lon/lat (LonLat or UTM inverse, core/Projections.cpp:200-232)
//   -> DEM height (biquintic FP32, geometry/DEMInterpolator.cpp:617-659)
//   -> geo2rdr Newton (geometry/detail/Geo2Rdr.icc:114-179), FP64
//   -> corrections, radar-grid checks, subswath mask (geocode/geocodeSlc.cpp:55-228)
//   -> per SLC block: 8x8 windowed-sinc with native-Doppler demodulation
//      (geocodeSlc.cpp:409-511, core/Sinc2dInterpolator.cpp:45-96),
//      then carrier reramp and flattening (geocodeSlc.cpp:298-394).
// Nothing here is a dense contraction, so no tensor cores; the kernel is
// bound by the FP64 pipe (geometry) and latency, not by HBM.
// Built twice: as is (plain launch, deramp, probe) and with
// GSLC_PERSISTENT_TU defined by gslc_persistent.cu (the persistent batched
// kernel), so that the two sets of kernel instances compile in parallel.
#include <algorithm>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <cuda_fp16.h>
#include "gslc_kernels.cuh"

namespace gslc {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    // std::complex<float> product for finite operands: (ac - bd, ad + bc)
    const float ac = fmul(a.x, b.x), bd = fmul(a.y, b.y), ad = fmul(a.x, b.y), bc = fmul(a.y, b.x);
    return make_float2(fsub(ac, bd), fadd(ad, bc));
}

// cos/sin of a large FP64 phase: reduce by 2*pi in FP64 (Cody-Waite with a
// two-term 2*pi), then evaluate in FP32.  Error ~1e-7 rad against the
// reference's float(cos(double)).
__device__ __forceinline__ float2 expi_fp64(double ph) {
    constexpr double INV_2PI = 0.15915494309189535;
    constexpr double TWO_PI_HI = 6.283185307179586;
    constexpr double TWO_PI_LO = 2.4492935982947064e-16;
    const double k = rint(ph * INV_2PI);
    double r = fma(-k, TWO_PI_HI, ph);
    r = fma(-k, TWO_PI_LO, r);
    float s, c;
    sincosf((float)r, &s, &c);
    return make_float2(c, s);
}

// DEM column coordinate from longitude for an EPSG:4326 DEM
// (geometry/DEMInterpolator.cpp:593-611 forward, :627-646 wrap and west edge).
// Returns false where the reference returns the reference height.
__device__ __forceinline__ bool dem_col_lonlat(const Dem& d, double lon, double& col) {
    double X = (lon * 180.0) / PI;
    if (X > 360 || X < -360) X = fmod(X, 360.0);
    if (X < -180) X += 360;
    if (X - 360 >= d.x_start) X -= 360;
    else if (X < d.x_start && X + 360 >= d.x_start) X += 360;
    else if (X < d.x_start) return false;
    col = (X - d.x_start) / d.dx;
    return true;
}

__device__ __forceinline__ double dem_row_lonlat(const Dem& d, double lat) {
    return (((lat * 180.0) / PI) - d.y_start) / d.dy;
}

// The CUDA DEM interpolator: LonLat::forward then the column, without the
// +-360 wrap of the CPU one (cuda/geometry/gpuDEMInterpolator.cu:149-204,
// cuda/core/gpuProjections.cu:108-117).
__device__ __forceinline__ double dem_col_lonlat_nowrap(const Dem& d, double lon) {
    return ((lon * 180.0) / PI - d.x_start) / d.dx;
}

// Both coordinates for a UTM DEM (forward projection per pixel).
__device__ __forceinline__ bool dem_coords_utm(const Dem& d, double lon, double lat, double& row, double& col) {
    double X, Y;
    if (!utm_forward(d.utm, lon, lat, X, Y)) return false;
    if (X < d.x_start) return false;
    row = (Y - d.y_start) / d.dy;
    col = (X - d.x_start) / d.dx;
    return true;
}

// Bounds checks (DEMInterpolator.cpp:648-655) and the order-6 biquintic
// spline in FP32 (core/Spline2dInterpolator.cpp:32-67).
__device__ double dem_spline(const Dem& d, double row, double col) {
    const double ref = 0.0;
    // truncation equals floor wherever the bounds below pass (row, col >= 2);
    // (col - j0) - 2 is col - icol, both steps exact for col >= 2.  The
    // integer parts and the fractions come from the bits (split_bits): a row
    // or column that is negative, NaN or at least 2^31 gives INT32_MAX and
    // fails the bounds, as its truncation does.
    uint64_t frow, fcol;
    const int irow = split_bits(row, frow), icol = split_bits(col, fcol);
    if (irow < 2 || irow >= d.length - 1) return ref;
    if (icol < 2 || icol >= d.width - 1) return ref;
    const int i0 = irow - 2, j0 = icol - 2;
    // rows i0 + 1 .. min(i0 + 6, length - 1) (the clamp below) must be on the device
    if (i0 + 1 < d.avail_lo || min(i0 + 6, d.length - 1) > d.avail_hi) {
        if (d.err) atomicOr(d.err, 8);
    }
    // (float)(col - icol) and (float)(row - irow)
    const float xx = fixed64_to_float(fcol);
    const float yy = fixed64_to_float(frow);
    int cidx[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) cidx[j] = min(max(j0 + j, 0), d.width - 2) + 1;
    float HC[6], A[6], R[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const int indi = min(max(i0 + i, 0), d.length - 2) + 1;
        const float* rowp = d.data + (int64_t)indi * d.stride;
#pragma unroll
        for (int j = 0; j < 6; ++j) A[j] = __ldg(rowp + cidx[j]);
        init_spline6(A, R, d.sc);
        HC[i] = spline6_at(xx, A, R);
    }
    init_spline6(HC, R, d.sc);
    return (double)spline6_at(yy, HC, R);
}

// The same bounds and window with the CUDA interpolator's mixed-precision
// spline (cuda/core/gpuSpline2dInterpolator.cu:119-145; the DEM reference
// height is 0).
__device__ double dem_spline_gpu(const Dem& d, double row, double col) {
    const int irow = (int)floor(row), icol = (int)floor(col);
    if (irow < 2 || irow >= d.length - 1) return 0.0;
    if (icol < 2 || icol >= d.width - 1) return 0.0;
    const int i0 = (int)row - 2, j0 = (int)col - 2;
    const double xs = dsub(col, (double)j0), ys = dsub(row, (double)i0);
    int cidx[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) cidx[j] = min(max(j0 + j, 0), d.width - 2) + 1;
    float HC[6], A[6], R[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const int indi = min(max(i0 + i, 0), d.length - 2) + 1;
        const float* rowp = d.data + (int64_t)indi * d.stride;
#pragma unroll
        for (int j = 0; j < 6; ++j) A[j] = __ldg(rowp + cidx[j]);
        init_spline6_gpu(A, R, d.sc);
        HC[i] = spline6_at_gpu(xs, A, R);
    }
    init_spline6_gpu(HC, R, d.sc);
    return (double)spline6_at_gpu(ys, HC, R);
}

template <bool RASTER>
__device__ __forceinline__ double dem_height(const Dem& d, double row, double col) {
    return RASTER ? dem_spline_gpu(d, row, col) : dem_spline(d, row, col);
}


// geometry/detail/Geo2Rdr.icc:50-112 (coarse search when the initial guess is
// outside the orbit)
__device__ bool update_aztime(const GeoParams& p, V3 xyz, double& t) {
    const double tstart = p.orbit.t0, tend = p.orbit.t_end;
    const double dt = (tend - tstart) / 14;
    double r_closest = 1e16, t_closest = -1000.;
    for (int k = 0; k < 15; ++k) {
        const double tt = tstart + k * dt;
        if (tt < tstart || tt > tend) continue;
        V3 pos, vel;
        orbit_eval(p.orbit, tt, pos, vel);
        const V3 rvec = vsub(xyz, pos);
        if (k == 0 && ((p.look_side == -1) != (vdot(vcross(rvec, vel), pos) > 0.))) return false;
        const double r = vnorm(rvec);
        if (r < r_closest) { r_closest = r; t_closest = tt; }
    }
    t = (t_closest < 0.) ? 0.5 * (tstart + tend) : t_closest;
    return true;
}

// geometry/detail/Geo2Rdr.icc:114-179 with geometry/geometry.cpp:241-251
// (deltaRange = 1e-8 as passed by geocodeSlc.cpp:120-123; the raster
// geocoder passes its delta_range argument).  With a
// zero image-grid Doppler the slant range enters only the returned iterate,
// so it is formed once, after convergence.
__device__ bool geo2rdr(const GeoParams& p, const double* seg, V3 xyz, double& t, double& R) {
    const double dr = p.dop_dr;
    t = p.t_mid;
    const bool first_shared = p.t_mid_in_orbit;
    if (!p.t_mid_in_orbit && !update_aztime(p, xyz, t)) return false;
    const bool dop_data = p.img_dop.have_data;
    const bool dop_const = !dop_data && (dbits(p.img_dop.ref_value) & DMAG) == 0;   // ref_value == 0.0
    if (p.maxiter < 1) return false;
    // the segment tables hold the Hermite pieces; with a Legendre orbit every
    // iteration interpolates the state vectors as the reference does
    const bool seg_path = dop_const && !p.orbit.legendre;
    if (seg_path && first_shared) {
        // iteration 0 at sensingMid with the shared state: the look-side
        // test (rvec x vel) . pos > 0 as rvec . (vel x pos), the step with
        // 1/|vel|^2 (within an ulp of the quotient)
        // (the sign and |dt| < thr tests on the bits, as in the Newton loop)
        const V3 rvec = vsub(xyz, p.pos0);
        const int64_t side = dkey(vdot(rvec, p.n0));
        if ((p.look_side == -1) != (side > 0 && side <= DKEY_INF)) return false;
        const double dt = -vdot(rvec, p.vel0) * p.inv_vv0;
        if ((dbits(dt) & DMAG) < p.thr_bits) {
            R = vnorm(rvec);
            return true;
        }
        return p.maxiter > 1 && geo2rdr_zero_doppler_seg(p.orbit, seg, xyz, p.thr, p.maxiter, t, dt, R);
    }
    const double half_wvl = 0.5 * p.rg_wvl;
    double dt = 0.0;
    for (int i = 0; i < p.maxiter; ++i) {
        t -= dt;
        V3 pos, vel;
        if (i == 0 && first_shared) {
            pos = p.pos0;
            vel = p.vel0;
        } else {
            if (!(t >= p.orbit.t0 && t <= p.orbit.t_end)) return false;  // FillNaN -> no convergence
            orbit_eval(p.orbit, t, pos, vel);
        }
        const V3 rvec = vsub(xyz, pos);
        if (i == 0 && ((p.look_side == -1) != (vdot(vcross(rvec, vel), pos) > 0.))) return false;
        if (seg_path) {
            // fdop == 0 and fdopder == 0 exactly: fn = rvec.vel, fn' = -vel.vel;
            // iterations after this one run on the segment tables
            dt = vdot(rvec, vel) / (-vdot(vel, vel));
            if (fabs(dt) < p.thr) {
                R = vnorm(rvec);
                return true;
            }
            return geo2rdr_zero_doppler_seg(p.orbit, seg, xyz, p.thr, p.maxiter, t, dt, R);
        }
        R = vnorm(rvec);
        if (dop_data && p.img_dop.bounds_error &&
            !(lut_contains(p.img_dop, t, R) && lut_contains(p.img_dop, t, R + dr)))
            return false;
        const double dopfact = vdot(rvec, vel);
        const double c1 = -vdot(vel, vel);
        const double fdop = half_wvl * lut_eval(p.img_dop, t, R);
        const double fdopder = (half_wvl * lut_eval(p.img_dop, t, R + dr) - fdop) / dr;
        const double fn = dopfact - fdop * R;
        const double c2 = (fdop / R) + fdopder;
        const double fnprime = c1 + c2 * dopfact;
        dt = fn / fnprime;
        if (fabs(dt) < p.thr) return true;
    }
    return false;
}

// The same Newton path in float-float.  Iteration 0 uses the shared FP64
// state at sensingMid; later iterations run on the float-pair segment tables
// (Orbit::seg_ff) in double-word FP32 (~2^-44 relative): the residual is the
// pixel's degree-13 polynomial fn(w) (coefficients D.b_k - h_k for k <= 6,
// D = xyz - P_ref formed in FP64 on segment entry, -h_k above), the step is
// -fn.G(w), and the segment coordinate w is tracked as a double word.  The
// FP64 pipe carries only the first iterate, segment entries and the final
// time and slant range.  Used when the image-grid Doppler is zero (the NISAR
// GSLC convention); otherwise the FP64 path runs.
__device__ __forceinline__ ff ld_ff(const float2* q) {
    const float2 v = __ldg(q);
    return {v.x, v.y};
}

__device__ bool geo2rdr_ff(const GeoParams& p, V3 xyz, double& t, double& R) {
    const Orbit& o = p.orbit;
    // iteration 0: t = sensingMid, shared position/velocity (FP64)
    t = p.t_mid;
    {
        const V3 rvec = vsub(xyz, p.pos0);
        const int64_t side = dkey(vdot(rvec, p.n0));
        if ((p.look_side == -1) != (side > 0 && side <= DKEY_INF)) return false;
        const double dt = -vdot(rvec, p.vel0) * p.inv_vv0;
        if ((dbits(dt) & DMAG) < p.thr_bits) {
            R = vnorm(rvec);
            return true;
        }
        t -= dt;
    }
    const float thr = (float)p.thr;
    const ff inv_sp = ff_from_double(o.inv_spacing);
    const int nh = o.seg_nh, ng = o.seg_ng;
    int j = -1;
    double tj = 0.0;                    // start time of segment j: t = tj + (w + 0.5) spacing
    ff w = {0.f, 0.f}, D[3], cf[7];
    const float2* c = o.seg_ff;
    for (int i = 1; i < p.maxiter; ++i) {
        const float wf = w.hi + w.lo;
        // entering or leaving a segment, and on the first and last segment
        // (the orbit's time span): time, span check and w from FP64
        if (j <= 0 || j >= o.n - 2 || !(wf >= -0.5f && wf < 0.5f)) {
            if (j >= 0) t = tj + ((double)w.hi + (double)w.lo + 0.5) * o.spacing;
            const int64_t kt = dkey(t);                         // the span test on order keys
            if (!(kt >= dkey(o.t0) && kt <= dkey(o.t_end))) return false;    // FillNaN -> no convergence
            // orbit_piece(o, t) truncated from the bits (t >= t0 here) and
            // the segment start times from the tables, as the FP64 path
            uint64_t fb;
            int pc = split_bits((t - o.t0) * o.inv_spacing + 1, fb) - 2;
            pc = pc < 0 ? 0 : (pc > o.n - 4 ? o.n - 4 : pc);
            const double tidx = __ldg(o.seg + (int64_t)pc * SEG_STRIDE + SEG_T);
            double w64 = (t - tidx) * o.inv_spacing - 1.5;
            const int jn = orbit_segment(o, pc, w64);
            w = ff_from_double(w64);
            if (jn != j) {
                j = jn;
                c = o.seg_ff + (int64_t)j * SEGFF_STRIDE;
                const double* pref = o.seg + (int64_t)j * SEG_STRIDE;
                tj = __ldg(pref + SEG_T);
                D[0] = ff_from_double(xyz.x - __ldg(pref + 0));
                D[1] = ff_from_double(xyz.y - __ldg(pref + 1));
                D[2] = ff_from_double(xyz.z - __ldg(pref + 2));
#pragma unroll
                for (int k = 0; k < 7; ++k) {
                    const ff dv = ff_add(ff_add(ff_mul(D[0], ld_ff(c + SEGFF_B + k)), ff_mul(D[1], ld_ff(c + SEGFF_B + 7 + k))),
                                         ff_mul(D[2], ld_ff(c + SEGFF_B + 14 + k)));
                    cf[k] = k <= nh ? ff_add(dv, ff_neg(ld_ff(c + SEGFF_H + k))) : dv;
                }
            }
        }
        ff fn = cf[6];
        if (nh > 6) {
            fn = ff_neg(ld_ff(c + SEGFF_H + nh));
            for (int k = nh - 1; k >= 7; --k) fn = ff_fma(fn, w, ff_neg(ld_ff(c + SEGFF_H + k)));
            fn = ff_fma(fn, w, cf[6]);
        }
#pragma unroll
        for (int k = 5; k >= 0; --k) fn = ff_fma(fn, w, cf[k]);
        // G = 1/|vel|^2 only scales the step: in FP32 (relative error ~1e-7)
        // each step changes by that fraction, which the next float-float
        // residual corrects (the iteration contracts by ~0.1 per step)
        float g = __ldg(c + SEGFF_G + ng).x;
        for (int k = ng - 1; k >= 0; --k) g = fmaf(g, w.hi, __ldg(c + SEGFF_G + k).x);
        const ff dt = ff_neg(ff_mul_f(fn, g));
        if (fabsf(dt.hi) < thr) {
            t = tj + ((double)w.hi + (double)w.lo + 0.5) * o.spacing;
            double r[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                ff acc = ld_ff(c + SEGFF_A + d * 8 + 6);
                if (o.seg_a7) acc = ff_fma(ld_ff(c + SEGFF_A + d * 8 + 7), w, acc);
#pragma unroll
                for (int k = 5; k >= 0; --k) acc = ff_fma(acc, w, ld_ff(c + SEGFF_A + d * 8 + k));
                r[d] = ff_to_double(ff_add(D[d], ff_neg(acc)));
            }
            R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            return true;
        }
        w = ff_add(w, ff_neg(ff_mul(dt, inv_sp)));
    }
    return false;
}

// product/SubSwaths.cpp:58-96
__device__ int subswath_of(const GeoParams& p, int az, int rg) {
    if (rg < 0 || rg >= p.subsw_wid || az < 0 || az >= p.subsw_len) return 0;
    if (p.subsw_n == 0) return 1;
    for (int s = 0; s < p.subsw_n; ++s) {
        const int32_t* v = p.subsw + ((int64_t)s * p.subsw_len + az) * 2;
        if (rg >= __ldg(v) && rg < __ldg(v + 1)) return s + 1;
    }
    return 0;
}

// geocodeSlc.cpp:409-511 for one pixel and one block: 9x9 chip demodulated
// by the native Doppler, Sinc2d over it (Sinc2dInterpolator.cpp:45-96), then
// the Doppler added back.  Sum order is the reference's (i outer, j inner).
__device__ __forceinline__ float2 ld_sample(const float2* q) { return __ldg(q); }
__device__ __forceinline__ float2 ld_sample(const __half2* q) {
    // complex32: float16 -> float32 is exact, as numpy's astype
    return __half22float2(__ldg(q));
}

// Sinc2dInterpolator's integer position and table phase of x = 4 + frac:
// i = floor(x), f = min(max(0, int((x - i) * SINC_SUB)), SINC_SUB - 1).  For
// x in [4, 8) both are bit fields of x (x = 4 (1 + m 2^-52): i = 4 + m >> 50
// and, for i = 4, (x - 4) SINC_SUB = m 2^-37, so f = m >> 37); other x take
// the FP64 form.
__device__ __forceinline__ void sinc_index(double x, int& i, int& f) {
    const uint64_t b = dbits(x);
    if ((b >> 52) == 0x401) {
        const uint64_t m = b & 0xfffffffffffffull;
        i = 4 + (int)(m >> 50);
        f = (int)((m >> 37) & (uint64_t)(SINC_SUB - 1));
        return;
    }
    i = (int)floor(x);
    f = min(max(0, (int)((x - i) * SINC_SUB)), SINC_SUB - 1);
}

// The chip sum at integer positions ix, iy (3 or 4) and table phases ifx,
// ify; fracAz_f is (float)fracAz, the demodulation's phase argument.
template <typename S>
__device__ __noinline__ float2 sinc_chip(const GeoParams& p, const S* __restrict__ rdr, int intAz, int intRg, int ix, int iy,
                            int ifx, int ify, float fracAz_f, float doppFreq) {
    float kx[8], ky[8];
    const float4* kxp = reinterpret_cast<const float4*>(p.sinc + ifx * SINC_LEN);
    const float4* kyp = reinterpret_cast<const float4*>(p.sinc + ify * SINC_LEN);
    {
        float4 a = __ldg(kxp), b = __ldg(kxp + 1), c = __ldg(kyp), d = __ldg(kyp + 1);
        kx[0] = a.x; kx[1] = a.y; kx[2] = a.z; kx[3] = a.w; kx[4] = b.x; kx[5] = b.y; kx[6] = b.z; kx[7] = b.w;
        ky[0] = c.x; ky[1] = c.y; ky[2] = c.z; ky[3] = c.w; ky[4] = d.x; ky[5] = d.y; ky[6] = d.z; ky[7] = d.w;
    }
    const bool demod = doppFreq != 0.f;
    // demodulation phasors for row offsets m = 0..4 (doppPhase = doppFreq*m)
    float dc[5], ds[5];
    if (demod) {
#pragma unroll
        for (int m = 0; m < 5; ++m) sincosf(doppFreq * (float)m, &ds[m], &dc[m]);
    }
    // chip row r9 = iy + 4 - i maps to radar row intAz + iy - i; col c9 = ix + 4 - j
    const S* base = rdr + (int64_t)(intAz + iy) * p.inW + (intRg + ix);
    float sre = 0.f, sim = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const S* rowp = base - (int64_t)i * p.inW;
        float2 dv = make_float2(1.f, 0.f);
        if (demod) {
            const int m = iy - i;
            const int am = m < 0 ? -m : m;
            // doppVal = (cos(phase), -sin(phase)), phase = doppFreq * m
            dv = make_float2(dc[am], m < 0 ? ds[am] : -ds[am]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float2 a = ld_sample(rowp - j);
            if (demod) a = cmul(a, dv);
            sre = fadd(sre, fmul(fmul(a.x, ky[i]), kx[j]));
            sim = fadd(sim, fmul(fmul(a.y, ky[i]), kx[j]));
        }
    }
    // A non-finite chip sample turns both parts of the reference's complex
    // products into NaN (x*0 with x = inf or NaN).
    if (!isfinite(sre) || !isfinite(sim)) return make_float2(CUDART_NAN_F, CUDART_NAN_F);
    float2 cval = make_float2(sre, sim);
    if (demod) {
        float s, c;
        sincosf(doppFreq * fracAz_f, &s, &c);
        cval = cmul(cval, make_float2(c, s));
    }
    return cval;
}

template <typename S>
__device__ float2 sinc_pixel(const GeoParams& p, const S* __restrict__ rdr, int intAz, int intRg,
                             double fracAz, double fracRg, float doppFreq) {
    int ix, iy, ifx, ify;
    sinc_index(4.0 + fracRg, ix, ifx);
    sinc_index(4.0 + fracAz, iy, ify);
    if (ix < 3 || ix > 4 || iy < 3 || iy > 4) return make_float2(0.f, 0.f);
    return sinc_chip(p, rdr, intAz, intRg, ix, iy, ifx, ify, (float)fracAz, doppFreq);
}

// block b of the request, in its sample format
__device__ __forceinline__ float2 sinc_block(const GeoParams& p, int b, int intAz, int intRg, double fracAz,
                                             double fracRg, float doppFreq) {
    if (p.rdr_c32) return sinc_pixel(p, reinterpret_cast<const __half2*>(p.rdr[b]), intAz, intRg, fracAz, fracRg, doppFreq);
    return sinc_pixel(p, p.rdr[b], intAz, intRg, fracAz, fracRg, doppFreq);
}

// The same with the table phases of fractions in 64-bit fixed point
// (split_bits): 4 + frac is exact in [4, 5) whenever the chip is
// interpolated (the fraction's last bit is at least the ulp of an index
// >= 4), so the integer position is 4 and the table phase the fraction's
// top 13 bits (sinc_index), without the FP64 additions.
__device__ __forceinline__ float2 sinc_block_fixed(const GeoParams& p, int b, int intAz, int intRg, int ify, int ifx,
                                                   float fracAz_f, float doppFreq) {
    if (p.rdr_c32)
        return sinc_chip(p, reinterpret_cast<const __half2*>(p.rdr[b]), intAz, intRg, 4, 4, ifx, ify, fracAz_f,
                         doppFreq);
    return sinc_chip(p, p.rdr[b], intAz, intRg, 4, 4, ifx, ify, fracAz_f, doppFreq);
}

// float32 -> float16 bits as numpy's astype(float16): round to nearest even
// (overflow to infinity), and NaN as sign | 0x7c00 | the top mantissa bits
// (never the infinity pattern)
__device__ __forceinline__ unsigned short f32_to_f16_bits(float x) {
    if (isnan(x)) {
        const unsigned int u = __float_as_uint(x);
        unsigned short h = (unsigned short)(((u >> 16) & 0x8000u) | 0x7c00u | ((u & 0x7fffffu) >> 13));
        if ((h & 0x3ffu) == 0) h |= 1u;
        return h;
    }
    return __half_as_ushort(__float2half_rn(x));
}

// output pixel k of block b in the request's output format
__device__ __forceinline__ void store_geo(const GeoParams& p, int b, int64_t k, float2 v) {
    if (p.geo_fmt == 0) {
        p.geo[b][k] = v;
    } else if (p.geo_fmt == 1) {
        const unsigned int w = (unsigned int)f32_to_f16_bits(v.x) | ((unsigned int)f32_to_f16_bits(v.y) << 16);
        reinterpret_cast<unsigned int*>(p.geo[b])[k] = w;
    } else {
        // truncate_mantissa: keep the sign, exponent and mant_bits mantissa bits
        const unsigned int m = 0xffffffffu << (23 - p.mant_bits);
        p.geo[b][k] = make_float2(__uint_as_float(__float_as_uint(v.x) & m), __uint_as_float(__float_as_uint(v.y) & m));
    }
}

// cuda/product/SubSwaths.h:177-205 (ViewSubSwaths::contains): no subswaths
// means everything is contained, tested before the bounds.
__device__ bool subswath_contains_gpu(const GeoParams& p, int az, int rg) {
    if (p.subsw_n == 0) return true;
    if (az < 0 || az >= p.subsw_len || rg < 0 || rg >= p.subsw_wid) return false;
    for (int s = 0; s < p.subsw_n; ++s) {
        const int32_t* v = p.subsw + ((int64_t)s * p.subsw_len + az) * 2;
        if (rg >= __ldg(v) && rg < __ldg(v + 1)) return true;
    }
    return false;
}

// Block shape: 32 x 8 threads.  A tile is 32 geogrid columns x 8*PPT
// lines; thread (tx, ty) geocodes lines ty, ty + 8, ... of column tx, so a
// warp stores 32 consecutive pixels of one line.
constexpr int GBX = 32, GBY = 8;

// ---- orbit tables in shared memory ----------------------------------------
// The Newton segment tables of the request (Orbit::seg, 608 B per
// state-vector interval) are brought into shared memory by one bulk
// asynchronous copy (cp.async.bulk, completion counted in bytes on an
// mbarrier) issued by one thread when the tile starts; it overlaps the
// tile's ground-point work and is waited for before the first Newton
// iteration.  Orbits whose tables exceed SEG_SMEM read them from global
// memory.  The wait is bounded: the copy must land within
// GeoParams::stage_wait SM clocks of its issue (a deadline, checked before
// each poll); a thread whose wait runs out reads the global tables, raises
// error bit 1 (GSLC_ETIMEOUT on the host) and the block stages nothing more.  Before the
// block finishes, one thread waits (bounded again) for a copy still in
// flight, so that the copy never writes shared memory the block has left;
// if that wait runs out too, error bit 2 is raised.
constexpr int SEG_SMEM = 4096;   // doubles (32 KiB): orbits of up to 54 state vectors

struct OrbitStage {
    double* buf;          // shared, 16-byte aligned
    uint64_t* bar;        // shared mbarrier
    int* off;             // shared flag: a wait ran out, stage nothing more
    uint32_t phase;       // parity of the copy to wait for
    int issued;           // a copy of this request's tables was issued
    long long deadline;   // SM clock by which the copy must have landed
    int* landed;          // shared flag: a wait saw this copy land (later waits on it succeed at once)
};

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
    return (uint32_t)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ uint32_t seg_bytes(const GeoParams& p) {
    return (uint32_t)((p.orbit.n - 1) * SEG_STRIDE * sizeof(double));
}

__device__ __forceinline__ bool seg_fits(const GeoParams& p) {
    return !p.orbit.legendre && p.orbit.n - 1 <= SEG_SMEM / SEG_STRIDE;
}

// one thread, once per block
__device__ __forceinline__ void stage_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one thread: the copy of p's segment tables into buf (the caller checked
// seg_fits; source and size are multiples of 16 bytes)
__device__ __forceinline__ void stage_issue(const GeoParams& p, double* buf, uint64_t* bar) {
    const uint32_t bytes = seg_bytes(p);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(buf)), "l"(p.orbit.seg), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred P;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, P;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// wait for a copy, at most `limit` SM clocks
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

// every thread: true when the staged tables can be read.  Past the deadline
// the wait has run out whether or not the copy landed meanwhile, unless an
// earlier wait on the same copy (a thread of this or of an earlier tile of
// the request) saw it land.
__device__ __forceinline__ bool stage_ready(const OrbitStage& st, const GeoParams& p) {
    if (!st.issued) return false;
    if (*(volatile int*)st.landed) return true;
    while (clock64() <= st.deadline)
        if (mbar_try_wait(st.bar, st.phase)) {
            *(volatile int*)st.landed = 1;
            return true;
        }
    atomicOr(p.err, 2);
    *st.off = 1;
    return false;
}

// one thread, before the block finishes: the copy of parity `parity` has
// landed (immediate when a wait already saw it), at most STAGE_WAIT_DEFAULT
// clocks
__device__ __forceinline__ void stage_drain(uint64_t* bar, uint32_t parity, int32_t* err) {
    if (!mbar_wait_bounded(bar, parity, STAGE_WAIT_DEFAULT)) atomicOr(err, 4);
}

// ---- tile fit of the projection inverse (UTM geogrids) --------------------
// Over one tile (at most 1 km on a side) the map from (column, line) to the
// DEM coordinates of the point, to lonLatToXyz(lon, lat, 0) and to the
// ellipsoid normal is smooth to far below the rounding of its exact
// evaluation: a bicubic Lagrange interpolant through 4 x 4 node pixels has a
// truncation error below 1e-16 rad (3e-10 m) there, so it stands in for the
// per-pixel UTM inverse (core/Projections.cpp:200-232), the DEM coordinate
// arithmetic (geometry/DEMInterpolator.cpp:593-646) and the trigonometry of
// Ellipsoid::lonLatToXyz (core/Ellipsoid.h:177-190).  The nodes are evaluated
// exactly; the interpolation adds a few ulps of rounding (coordinates) and
// ~3e-9 m (positions).  Tiles where a node fails the inverse, or where nodes
// disagree on the DEM branch (west edge, 360-degree wrap, DEM forward
// projection), take the exact per-pixel path.
constexpr int FIT_Q = 8;   // dem row, dem col, xyz0[3], normal[3]

template <int N>
struct FitNodes {
    int v[4];
    constexpr FitNodes() : v{0, (N - 1 + 1) / 3, (2 * (N - 1) + 1) / 3, N - 1} {}
};

struct FitWeights {
    double xs[GBX];            // column / (GBX - 1), the variable of the per-line cubic
    double m[3][3];            // column-node differences -> cubic coefficients 1..3
    double y8[8][4], y16[16][4], y32[32][4];
};

// Inverse of V[i][k] = x_i^(k+1) (i, k = 0..2) for the three column nodes
// after the first, x_i = node / (GBX - 1): the cubic through the node
// values g_0..g_3 of one line is g_0 + c1 x + c2 x^2 + c3 x^3 with
// c = V^-1 (g_1 - g_0, g_2 - g_0, g_3 - g_0).
constexpr void fit_cubic_matrix(double (&m)[3][3]) {
    const FitNodes<GBX> nd;
    double v[3][3] = {};
    for (int i = 0; i < 3; ++i) {
        const double x = (double)nd.v[i + 1] / (double)(GBX - 1);
        v[i][0] = x;
        v[i][1] = x * x;
        v[i][2] = x * x * x;
    }
    const double det = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]) -
                       v[0][1] * (v[1][0] * v[2][2] - v[1][2] * v[2][0]) +
                       v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            // cofactor of v[j][i] (transposed), over det
            const int r0 = j == 0 ? 1 : 0, r1 = j == 2 ? 1 : 2;
            const int c0 = i == 0 ? 1 : 0, c1 = i == 2 ? 1 : 2;
            const double minor = v[r0][c0] * v[r1][c1] - v[r0][c1] * v[r1][c0];
            m[i][j] = (((i + j) & 1) ? -minor : minor) / det;
        }
}

template <int N>
constexpr void fit_weights(double (&w)[N][4]) {
    const FitNodes<N> nd;
    for (int t = 0; t < N; ++t)
        for (int i = 0; i < 4; ++i) {
            double v = 1.0;
            for (int k = 0; k < 4; ++k)
                if (k != i) v = v * (double)(t - nd.v[k]) / (double)(nd.v[i] - nd.v[k]);
            w[t][i] = v;
        }
}

constexpr FitWeights make_fit_weights() {
    FitWeights f{};
    for (int t = 0; t < GBX; ++t) f.xs[t] = (double)t / (double)(GBX - 1);
    fit_cubic_matrix(f.m);
    fit_weights<8>(f.y8);
    fit_weights<16>(f.y16);
    fit_weights<32>(f.y32);
    return f;
}

__constant__ FitWeights c_fit = make_fit_weights();

template <int TY>
__device__ __forceinline__ double fit_wy(int r, int j) {
    if (TY == 8) return c_fit.y8[r][j];
    if (TY == 16) return c_fit.y16[r][j];
    return c_fit.y32[r][j];
}

// DEM column for an EPSG:4326 DEM as dem_col_lonlat, with the branch taken:
// 0 none, 1 -360, 2 +360, 3 west of the DEM (reference height), +4 if the
// 360-degree fmod applied.
__device__ __forceinline__ int dem_col_lonlat_branch(const Dem& d, double lon, double& col) {
    double X = (lon * 180.0) / PI;
    int br = 0;
    if (X > 360 || X < -360) { X = fmod(X, 360.0); br = 4; }
    if (X < -180) X += 360;
    if (X - 360 >= d.x_start) { X -= 360; br += 1; }
    else if (X < d.x_start && X + 360 >= d.x_start) { X += 360; br += 2; }
    else if (X < d.x_start) return br + 3;
    col = (X - d.x_start) / d.dx;
    return br;
}

// Exact values of the fitted quantities at one node pixel; the DEM branch,
// or -1 where the UTM inverse fails.
template <bool RASTER>
__device__ int fit_node(const GeoParams& p, int pixel, int line, double* F) {
    const double x = dadd(p.gx0, dmul(p.gdx, (double)pixel + 0.5));
    const double y = dadd(p.gy0, dmul(p.gdy, (double)(line + p.geo_row0) + 0.5));
    const UtmCol c = utm_inverse_col(p.utm, x);
    if (!c.ok) return -1;
    const UtmRow r = utm_inverse_row(p.utm, y);
    const LonLatSC ll = utm_inverse_px(p.utm, r, c);
    double row = 0.0, col = 0.0;
    int br = 0;
    if (p.dem.have_raster) {
        if (p.dem.epsg_is_lonlat) {
            row = dem_row_lonlat(p.dem, ll.lat);
            if (RASTER) col = dem_col_lonlat_nowrap(p.dem, ll.lon);
            else br = dem_col_lonlat_branch(p.dem, ll.lon, col);
        } else {
            br = dem_coords_utm(p.dem, ll.lon, ll.lat, row, col) ? 0 : 3;
        }
    }
    const double re = p.ell_a / sqrt(1.0 - p.ell_e2 * (ll.slat * ll.slat));
    F[0] = row;
    F[1] = col;
    F[2] = re * ll.clat * ll.clon;
    F[3] = re * ll.clat * ll.slon;
    F[4] = (re * (1.0 - p.ell_e2)) * ll.slat;
    F[5] = ll.clat * ll.clon;
    F[6] = ll.clat * ll.slon;
    F[7] = ll.slat;
    return br;
}

template <bool FF, bool RASTER>
__device__ __forceinline__ void geocode_pixel(const GeoParams& p, const double* seg, int64_t k, bool ok, V3 xyz);

// One tile (tile column bx, tile line by) of one geocode request.
// RASTER selects the generic CUDA raster geocoder's per-pixel rules
// (cuda/geocode/Geocode.cu:87-172 and :203-287): DEM through the CUDA
// interpolator, corrections and native Doppler that do not contain the
// point mask it, no Doppler demodulation, carrier or flattening.
template <bool GEO_LONLAT, bool FF, bool RASTER, int PPT>
__device__ __forceinline__ void geocode_block(const GeoParams& p, int bx, int by, const OrbitStage& st) {
    constexpr int TY = GBY * PPT;
    __shared__ double s_col[4][GBX];
    __shared__ double s_row[5][TY];
    __shared__ int s_colok[GBX];
    __shared__ double s_F[16][FIT_Q];
    __shared__ int s_nb[16];
    __shared__ double s_G[TY][FIT_Q][4];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * GBX + tx;
    const int pixel = bx * GBX + tx;
    const int line0 = by * TY;
    const bool dem_ll = p.dem.have_raster && p.dem.epsg_is_lonlat;

    bool fit = false;
    if (!GEO_LONLAT && p.tile_fit && fabs(p.gdx) * (GBX - 1) <= 1000.0 && fabs(p.gdy) * (TY - 1) <= 1000.0) {
        constexpr FitNodes<GBX> nx;
        constexpr FitNodes<TY> ny;
        if (tid < 16) s_nb[tid] = fit_node<RASTER>(p, bx * GBX + nx.v[tid & 3], line0 + ny.v[tid >> 2], s_F[tid]);
        __syncthreads();
        fit = s_nb[0] >= 0;
#pragma unroll
        for (int n = 1; n < 16; ++n) fit = fit && s_nb[n] == s_nb[0];
        if (fit) {
            // the node values reduced over the line nodes, per tile line:
            // g_i = sum_j F[j][i][q] * wy[r][j] at the four column nodes, then
            // the line's cubic in x = column / (GBX - 1):
            // G[r][q] = (g_0, c1, c2, c3), c = m (g_1 - g_0, g_2 - g_0, g_3 - g_0).
            // The differences are exact (Sterbenz) for the slowly varying
            // quantities, so a pixel's value rounds once at its magnitude.
            for (int idx = tid; idx < TY * FIT_Q; idx += GBX * GBY) {
                const int r = idx / FIT_Q, q = idx % FIT_Q;
                double g[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    double a = 0.0;
#pragma unroll
                    for (int j = 0; j < 4; ++j) a = fma(s_F[j * 4 + i][q], fit_wy<TY>(r, j), a);
                    g[i] = a;
                }
                const double d1 = g[1] - g[0], d2 = g[2] - g[0], d3 = g[3] - g[0];
                s_G[r][q][0] = g[0];
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    s_G[r][q][k + 1] = fma(c_fit.m[k][0], d1, fma(c_fit.m[k][1], d2, c_fit.m[k][2] * d3));
            }
            __syncthreads();
        }
    }
    if (!fit) {
        if (ty == 0) {
            // pixel centre easting/longitude (geocodeSlc.cpp:103), same rounding as the reference
            const int pc = min(pixel, p.gw - 1);
            const double x = dadd(p.gx0, dmul(p.gdx, (double)pc + 0.5));
            if (GEO_LONLAT) {
                const double lon = (x * PI) / 180.0;          // LonLat::inverse (Projections.h:136-140)
                double sl, cl;
                sincos(lon, &sl, &cl);
                double col = 0.0;
                if (RASTER) {
                    s_colok[tx] = 1;
                    if (dem_ll) col = dem_col_lonlat_nowrap(p.dem, lon);
                } else {
                    s_colok[tx] = dem_ll ? (dem_col_lonlat(p.dem, lon, col) ? 1 : 0) : 1;
                }
                s_col[0][tx] = lon;
                s_col[1][tx] = sl;
                s_col[2][tx] = cl;
                s_col[3][tx] = col;
            } else {
                const UtmCol c = utm_inverse_col(p.utm, x);
                s_col[0][tx] = c.Ce;
                s_col[1][tx] = c.shi;
                s_col[2][tx] = c.chi;
                s_colok[tx] = c.ok;
            }
        } else if (ty == 1 && tx < TY) {
            const int lr = min(line0 + tx, p.gl - 1) + p.geo_row0;
            const double y = dadd(p.gy0, dmul(p.gdy, (double)lr + 0.5));   // geocodeSlc.cpp:100
            if (GEO_LONLAT) {
                const double lat = (y * PI) / 180.0;
                double sl, cl;
                sincos(lat, &sl, &cl);
                s_row[0][tx] = lat;
                s_row[1][tx] = sl;
                s_row[2][tx] = cl;
                s_row[3][tx] = p.ell_a / sqrt(1.0 - p.ell_e2 * (sl * sl));    // rEast (Ellipsoid.h:117-120)
                s_row[4][tx] = dem_ll ? dem_row_lonlat(p.dem, lat) : 0.0;
            } else {
                const UtmRow r = utm_inverse_row(p.utm, y);
                s_row[0][tx] = r.Cn;
                s_row[1][tx] = r.sr;
                s_row[2][tx] = r.cr;
            }
        }
        __syncthreads();
    }
    if (pixel >= p.gw) return;
    const double* seg = stage_ready(st, p) ? st.buf : p.orbit.seg;
    const double xs = c_fit.xs[tx];
#pragma unroll 1
    for (int kk = 0; kk < PPT; ++kk) {
        const int r = ty + GBY * kk;       // tile line
        const int line = line0 + r;
        if (line >= p.gl) break;
        const int64_t k = (int64_t)line * p.gw + pixel;
        bool ok = true;
        V3 xyz;
        if (fit) {
            double f[FIT_Q];
#pragma unroll
            for (int q = 0; q < FIT_Q; ++q)
                f[q] = fma(fma(fma(s_G[r][q][3], xs, s_G[r][q][2]), xs, s_G[r][q][1]), xs, s_G[r][q][0]);
            double h = 0.0;
            if (p.dem.have_raster && (s_nb[0] & 3) != 3) h = dem_height<RASTER>(p.dem, f[0], f[1]);
            xyz = {fma(h, f[5], f[2]), fma(h, f[6], f[3]), fma(h, f[7], f[4])};
        } else if (GEO_LONLAT) {
            double h = 0.0;
            if (p.dem.have_raster) {
                if (dem_ll) {
                    if (s_colok[tx]) h = dem_height<RASTER>(p.dem, s_row[4][r], s_col[3][tx]);
                } else {
                    double row, col;
                    if (dem_coords_utm(p.dem, s_col[0][tx], s_row[0][r], row, col))
                        h = dem_height<RASTER>(p.dem, row, col);
                }
            }
            // lonLatToXyz (Ellipsoid.h:177-190) with the line's rEast and the sines/cosines above
            const double re = s_row[3][r], slat = s_row[1][r], clat = s_row[2][r];
            xyz = {(re + h) * clat * s_col[2][tx], (re + h) * clat * s_col[1][tx],
                   ((re * (1.0 - p.ell_e2)) + h) * slat};
        } else {
            ok = s_colok[tx];
            if (!ok) {
                if (!RASTER) atomicOr(p.err, 1);   // the raster geocoder does not check the inverse
            } else {
                UtmCol c;
                c.Ce = s_col[0][tx]; c.shi = s_col[1][tx]; c.chi = s_col[2][tx]; c.ok = 1;
                UtmRow rr;
                rr.Cn = s_row[0][r]; rr.sr = s_row[1][r]; rr.cr = s_row[2][r];
                const LonLatSC ll = utm_inverse_px(p.utm, rr, c);
                double h = 0.0;
                if (p.dem.have_raster) {
                    double row, col;
                    if (dem_ll) {
                        if (RASTER)
                            h = dem_height<true>(p.dem, dem_row_lonlat(p.dem, ll.lat), dem_col_lonlat_nowrap(p.dem, ll.lon));
                        else if (dem_col_lonlat(p.dem, ll.lon, col))
                            h = dem_spline(p.dem, dem_row_lonlat(p.dem, ll.lat), col);
                    } else if (dem_coords_utm(p.dem, ll.lon, ll.lat, row, col)) {
                        h = dem_height<RASTER>(p.dem, row, col);
                    }
                }
                xyz = lonlat_to_xyz_sc(p.ell_a, p.ell_e2, ll.slon, ll.clon, ll.slat, ll.clat, h);
            }
        }
        geocode_pixel<FF, RASTER>(p, seg, k, ok, xyz);
    }
}

// (R - r0) / dr, correctly rounded as the quotient, in Markstein's form
// (q0 = a/dr by the correctly rounded reciprocal, one FMA residual, one FMA
// correction: Markstein 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, sec. 4.9), without the division's longer FP64 sequence.
__device__ __forceinline__ double range_index(const GeoParams& p, double R) {
    const double a = R - p.rg_r0;
    const double q0 = a * p.rg_inv_dr;
    return fma(fma(-q0, p.rg_dr, a), p.rg_inv_dr, q0);
}

// Everything after the ground point: geo2rdr, corrections, masks, the
// radar-coordinate outputs, the sinc interpolation of every block, reramp
// and flattening, for output pixel k.
template <bool FF, bool RASTER>
__device__ __forceinline__ void geocode_pixel(const GeoParams& p, const double* seg, int64_t k, bool ok, V3 xyz) {
    bool valid = false;
    uint8_t mval = 255;
    double azc = CUDART_NAN, rgc = CUDART_NAN;
    double R_uncorr = 0.0;          // the uncorrected slant range, set where the pixel converges
    if (ok) {
        double t, R;
        bool conv;
        if (FF) conv = geo2rdr_ff(p, xyz, t, R);
        else conv = geo2rdr(p, seg, xyz, t, R);
        if (RASTER) {
            // Geocode.cu:126-171: corrections and native Doppler that do not
            // contain the point mask it; floor indices inside the radar grid
            bool masked = !conv;
            if (conv) {
                if (lut_contains(p.az_corr, t, R)) t += lut_eval(p.az_corr, t, R);
                else masked = true;
                if (lut_contains(p.sr_corr, t, R)) R += lut_eval(p.sr_corr, t, R);
                else masked = true;
                if (!lut_contains(p.nat_dop, t, R)) masked = true;
            }
            const double yv = (t - p.rg_t0) * p.rg_prf;
            const double xv = range_index(p, R);
            const int yi = (int)floor(yv), xi = (int)floor(xv);
            if (!masked && p.have_subsw && !subswath_contains_gpu(p, yi, xi)) masked = true;
            const bool outside = yi < 0 || yi >= p.rg_len || xi < 0 || xi >= p.rg_wid;
            if (!masked && !outside) {
                valid = true;
                azc = yv;
                rgc = xv;
                mval = 1;
            }
        } else if (conv) {
            if (!p.use_corr) R_uncorr = R;
            // (a table without data adds its reference value; adding zero is skipped)
            if (p.az_corr_on && lut_contains(p.az_corr, t, R)) t += lut_eval(p.az_corr, t, R);
            if (p.sr_corr_on && lut_contains(p.sr_corr, t, R)) R += lut_eval(p.sr_corr, t, R);
            const int64_t kt = dkey(t), kr = dkey(R);
            const bool in_grid = kt >= p.k_s_t0 && kr >= p.k_s_r0 && kt <= p.k_s_stop && kr <= p.k_s_end;
            if (in_grid && lut_contains(p.nat_dop, t, R)) {
                azc = (t - p.rg_t0) * p.rg_prf;
                rgc = range_index(p, R);
                valid = true;
                const int intAz = floor_int(azc), intRg = floor_int(rgc);
                const bool corners = !(intRg < 4 || intRg >= p.rg_wid - 4 || intAz < 4 || intAz >= p.rg_len - 4);
                if (p.have_subsw && p.mask) {
                    int m = subswath_of(p, intAz, intRg);
                    if (m != 0) {
                        if (subswath_of(p, intAz - 4, intRg - 4) == 0 || subswath_of(p, intAz - 4, intRg + 4) == 0 ||
                            subswath_of(p, intAz + 4, intRg - 4) == 0 || subswath_of(p, intAz + 4, intRg + 4) == 0)
                            m = 0;
                    }
                    mval = (uint8_t)m;
                } else if (corners) {
                    mval = 1;
                }
            }
        }
    }
    if (p.mask) p.mask[k] = mval;
    if (p.az_out) p.az_out[k] = azc;
    if (p.rg_out) p.rg_out[k] = rgc;

    if (RASTER) {
        // Geocode.cu:232-287: the sinc chip must lie 4 samples inside the
        // radar raster (the reference's block bounding box +-5 lines/samples
        // reduces to this), then Sinc2d over the undemodulated chip
        const bool inside = valid && !(rgc < 4.0 || azc < 4.0 || rgc >= (double)p.inW - 4.0 ||
                                       azc >= (double)p.inL - 4.0);
        if (!inside) {
            for (int b = 0; b < p.nblk; ++b) store_geo(p, b, k, make_float2(p.inv_blk[b], p.inv_blk[b]));
            return;
        }
        const int xi = (int)floor(rgc), yi = (int)floor(azc);
        const double fx = rgc - (double)xi, fy = azc - (double)yi;
        for (int b = 0; b < p.nblk; ++b) store_geo(p, b, k, sinc_block(p, b, yi, xi, fy, fx, 0.f));
        return;
    }
    const float2 invalid = make_float2(p.inv_re, p.inv_im);
    if (!valid) {
        for (int b = 0; b < p.nblk; ++b) store_geo(p, b, k, invalid);
        return;
    }
    // block-relative chip position (geocodeSlc.cpp:440-458, 335-348).
    // RgIndex = rgc - rg_first is exact, so for rgc >= rg_first its integer
    // part is trunc(rgc) - rg_first and its fraction that of rgc; below
    // rg_first, under 1, or with the sign bit set every form gives an integer
    // part under 4 or past the block, which skips the chip.  Both come from
    // the bits of rgc and azc (split_bits); likewise in azimuth.
    uint64_t frg, faz;
    const int64_t intRgB64 = (int64_t)split_bits(rgc, frg) - p.rg_first;
    const int64_t intAzB64 = (int64_t)split_bits(azc, faz) - p.az_first;
    bool interp = !(intRgB64 < 4 || intRgB64 >= p.inW - 4 || intAzB64 < 4 || intAzB64 >= p.inL - 4);
    const int intRgB = (int)intRgB64, intAzB = (int)intAzB64;
    static_assert(SINC_SUB == 8192, "table phase = top 13 bits of the fraction");
    const int ifx = (int)(frg >> 51), ify = (int)(faz >> 51);
    const float fracAz_f = fixed64_to_float(faz);   // (float)fracAz
    double rng = 0.0, az = 0.0;
    float dop = 0.f;
    if (interp) {
        rng = dadd(p.rg_r0, dmul(rgc, p.rg_dr));
        az = p.rg_t0 + azc * p.inv_prf;
        // the Doppler in FP32: it only sets the float phases of the chip's demodulation
        if (p.chip_dop) {
            // contains(az, rng) on the indices' keys; the table coordinates
            // (index - origin) * cells per index, the integer parts exact
            // (|difference| < 2^21 inside the table), one rounding each
            const int64_t ka = dkey(azc), kr = dkey(rgc);
            interp = ka >= p.cd_kaz_lo && ka <= p.cd_kaz_hi && kr >= p.cd_krg_lo && kr <= p.cd_krg_hi;
            if (interp) {
                const float naz = small_int_to_float((int32_t)(intAzB64 + p.az_first - p.cd_iaz));
                const float nrg = small_int_to_float((int32_t)(intRgB64 + p.rg_first - p.cd_irg));
                const float yf = fmaf(naz, p.cd_saz, (fracAz_f - p.cd_faz) * p.cd_saz);
                const float xf = fmaf(nrg, p.cd_srg, (fixed64_to_float(frg) - p.cd_frg) * p.cd_srg);
                dop = lut_bilinear_f32(p.nat_dop, xf, yf);
            }
        } else {
            interp = lut_contains_eval_f32(p.nat_dop, az, rng, dop);
        }
    }
    if (!interp) {
        for (int b = 0; b < p.nblk; ++b) store_geo(p, b, k, invalid);
        return;
    }
    // the chip's lines intAzB - 4 .. intAzB + 4 must be on the device
    if (intAzB - 4 < p.avail_az_lo || intAzB + 4 > p.avail_az_hi) atomicOr(p.err, 8);
    // Doppler in radians per line: eval * 2 * pi / prf (geocodeSlc.cpp:473-474)
    const float doppFreq = dop * p.two_pi_over_prf_f;
    // reramp + flatten phase (geocodeSlc.cpp:362-392)
    const double carrier = p.carriers_zero ? 0.0 : azrg_eval(p.rg_car, az, rng) + azrg_eval(p.az_car, az, rng);
    const double flat = p.flat_scale * (p.use_corr ? rng : R_uncorr);
    // 0.0 + carrier is carrier but for a -0.0 carrier, and either zero
    // skips the rotation below; the sums are otherwise the reference's
    double total = p.reramp ? carrier : 0.0;
    if (p.flatten) total = p.reramp ? total + flat : flat;
    if (p.carrier_out) p.carrier_out[k] = carrier;
    if (p.flatten_out) p.flatten_out[k] = flat;
    const bool rot = (dbits(total) & DMAG) != 0;    // total != 0.0
    float2 ph = make_float2(1.f, 0.f);
    if (rot) ph = expi_fp64(total);
    for (int b = 0; b < p.nblk; ++b) {
        float2 v = sinc_block_fixed(p, b, intAzB, intRgB, ify, ifx, fracAz_f, doppFreq);
        if (rot) v = cmul(v, ph);
        store_geo(p, b, k, v);
    }
}

// Two blocks per SM: the UTM variants fit 128 registers without spills
// (190 unbounded), doubling the warps that hide FP64 and float-float latency.
template <bool GEO_LONLAT, bool FF, bool RASTER, int PPT>
__global__ void __launch_bounds__(GBX * GBY, 2) geocode_kernel(const __grid_constant__ GeoParams p) {
    __shared__ __align__(128) double s_seg[SEG_SMEM];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_off, s_landed;
    // the float-float path reads only the piece tables
    const bool stage = !FF && seg_fits(p);
    const long long deadline = clock64() + p.stage_wait;
    if (stage && threadIdx.x == 0 && threadIdx.y == 0) {
        s_landed = 0;
        stage_init(&s_bar);
        stage_issue(p, s_seg, &s_bar);
    }
    // geocode_block synchronises the block before any thread waits
    const OrbitStage st{s_seg, &s_bar, &s_off, 0u, stage ? 1 : 0, deadline, &s_landed};
    geocode_block<GEO_LONLAT, FF, RASTER, PPT>(p, blockIdx.x, blockIdx.y, st);
    // thread (0, 0) always has pixels (tiles start inside the geogrid), so
    // it reaches this point; the block's shared memory outlives the copy
    if (stage && threadIdx.x == 0 && threadIdx.y == 0) stage_drain(&s_bar, 0u, p.err);
}

// Persistent form: blocks pop runs of tiles of any request in the batch from
// one counter until the batch is exhausted.  Requests keep their own
// parameters, so each request's output equals its plain call.
template <bool GEO_LONLAT, bool FF, int PPT>
__global__ void __launch_bounds__(GBX * GBY, 2) geocode_persistent(const __grid_constant__ BatchQueue q) {
    // The block's queue position and staging state are block-uniform and
    // live in shared memory, written by the lead thread between barriers:
    // nothing of the loop stays in registers across a tile's body, which
    // has the same register budget as the plain kernel's.
    __shared__ long long s_next, s_end, s_tile;
    __shared__ __align__(128) double s_seg[SEG_SMEM];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ int s_off;
    __shared__ int s_staged;    // items[] entry the block last prepared for
    __shared__ int s_issued;    // a copy for it was issued
    __shared__ uint32_t s_phase;   // parity of the next copy
    __shared__ int s_any;       // a copy was issued (the last one has parity s_phase ^ 1)
    __shared__ long long s_deadline;
    __shared__ int s_landed;    // a wait saw the current copy land
    const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
    if (lead) {
        s_off = 0;
        s_landed = 0;
        s_next = s_end = 0;
        s_staged = -1;
        s_issued = 0;
        s_phase = 0;
        s_any = 0;
        if (!FF) stage_init(&s_bar);
    }
    for (;;) {
        if (lead) {
            // the next tile of the block's current pop, or a new pop of tiles_per_pop
            if (s_next >= s_end) {
                s_next = (long long)atomicAdd(reinterpret_cast<unsigned long long*>(q.counter),
                                              (unsigned long long)q.tiles_per_pop);
                s_end = min(s_next + (long long)q.tiles_per_pop, q.n_tiles);
            }
            s_tile = s_next < q.n_tiles ? s_next++ : -1;
        }
        __syncthreads();
        const long long tile = s_tile;
        if (tile < 0) {
            // the block's shared memory outlives its last copy
            if (!FF && lead && s_any) stage_drain(&s_bar, s_phase ^ 1u, q.items[0].err);
            return;
        }
        // request owning the tile: last prefix start <= tile (warp-uniform search)
        int lo = 0, hi = q.n_items - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (q.tile_start[mid] <= tile) lo = mid;
            else hi = mid - 1;
        }
        const GeoParams& p = q.items[lo];
        const long long local = tile - q.tile_start[lo];
        const int tiles_x = (p.gw + GBX - 1) / GBX;
        // every thread finished the previous tile (barrier below), so the
        // tables of a new request may overwrite s_seg; after a wait ran out
        // (s_off) nothing more is staged and the new request reads its global
        // tables.  The lead thread decides; the others read its decision.
        if (!FF && lead && lo != s_staged) {
            s_staged = lo;
            s_issued = (!s_off && seg_fits(p)) ? 1 : 0;
            if (s_issued) {
                s_deadline = clock64() + p.stage_wait;
                s_landed = 0;
                stage_issue(p, s_seg, &s_bar);
                s_phase ^= 1u;
                s_any = 1;
            }
        }
        __syncthreads();
        // (the copy just issued, if any, has parity s_phase ^ 1)
        const OrbitStage st{s_seg, &s_bar, &s_off, s_phase ^ 1u, FF ? 0 : s_issued, s_deadline, &s_landed};
        geocode_block<GEO_LONLAT, FF, false, PPT>(p, (int)(local % tiles_x), (int)(local / tiles_x), st);
        if (q.done_flags) __threadfence();   // this thread's outputs before the tile count
        __syncthreads();
        if (q.done_flags && lead) {
            // the block finishing a request's last tile raises its flag
            const int r = q.item_request[lo];
            const unsigned long long old = atomicAdd(q.request_done + r, 1ull);
            if ((long long)old + 1 == q.request_tiles[r]) {
                __threadfence_system();
                *(volatile unsigned int*)(q.done_flags + r) = 1u;   // single writer
            }
        }
    }
}

#ifndef GSLC_PERSISTENT_TU
// The carrier on one radar line, in the reference's operation order
// (core/Poly2d.cpp:8-24, core/LUT2d.cpp:124-158): a Poly2d of range order 0
// is constant along the line; otherwise it is evaluated per sample.
struct CarrierLine {
    int mode;          // 0 zero, 1 constant on the line, 2 Poly2d per sample, 3 LUT2d per sample
    double val, yval;
};

__device__ __forceinline__ CarrierLine carrier_line(const AzRg& f, double az) {
    CarrierLine c{0, 0.0, 0.0};
    if (f.is_zero) return c;
    if (f.kind != 1) {
        c.mode = 3;
        return c;
    }
    c.yval = ddiv(dsub(az, f.poly.y_mean), f.poly.y_norm);
    if (f.poly.x_order == 0) {
        c.mode = 1;
        c.val = poly_eval_exact(f.poly, c.yval, 0.0);
    } else {
        c.mode = 2;
    }
    return c;
}

__device__ __noinline__ double carrier_sample(const AzRg& f, const CarrierLine& c, double az, double rg) {
    return c.mode == 2 ? poly_eval_exact(f.poly, c.yval, rg) : lut_eval_exact(f.lut, az, rg);
}

__device__ __forceinline__ double carrier_at(const AzRg& f, const CarrierLine& c, double az, double rg) {
    if (c.mode == 0) return 0.0;
    if (c.mode == 1) return c.val;
    return carrier_sample(f, c, az, rg);
}

// geocodeSlc.cpp:240-274: rdr *= exp(-i * float(rg_carrier + az_carrier)),
// the FP64 phase bit-for-bit in the reference's order, so that its float
// rounding agrees.  Grid: x covers a line in chunks of 1024 samples, y the
// lines (per-sample carriers) or tiles of DR_LINES lines (line-constant).
__host__ __device__ __forceinline__ bool carrier_line_constant(const AzRg& f) {
    return f.is_zero || (f.kind == 1 && f.poly.x_order == 0);
}

// e^(-i phase) of line i of the block (both carriers constant along lines)
__device__ __forceinline__ float2 deramp_line_phasor(const DerampParams& p, int64_t i) {
    const double az = dadd(p.rg_t0, ddiv((double)(i + p.az_first), p.rg_prf));
    const CarrierLine lr = carrier_line(p.rg_car, az), la = carrier_line(p.az_car, az);
    const float phase = (float)dadd(lr.mode ? lr.val : 0.0, la.mode ? la.val : 0.0);
    float sn, cs;
    sincosf(phase, &sn, &cs);
    return make_float2(cs, -sn);
}

// Carriers constant along lines: tiles of DR_LINES lines x 1024 samples per
// block.  Lane l of every warp forms the phasor of the tile's line l (the
// FP64 carrier and its float phase, as the per-sample form), so the
// phasors of 32 lines cost one evaluation's latency; each warp then streams
// its 128-sample slice of the tile's lines, four lines' loads in flight
// before their stores (in place, each sample is read and written by one
// thread).
constexpr int DR_LINES = 32;

__global__ void __launch_bounds__(256) deramp_lines_kernel(const __grid_constant__ DerampParams p) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t c0 = (int64_t)blockIdx.x * 1024 + warp * 128 + lane;
    for (int64_t i0 = (int64_t)blockIdx.y * DR_LINES; i0 < p.inL; i0 += (int64_t)gridDim.y * DR_LINES) {
        const float2 rot_l = i0 + lane < p.inL ? deramp_line_phasor(p, i0 + lane) : make_float2(1.f, 0.f);
        const int nl = (int)(p.inL - i0 < DR_LINES ? p.inL - i0 : DR_LINES);
        for (int l0 = 0; l0 < nl; l0 += 4) {
            float2 v[4][4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const int64_t i = i0 + l0 + a;
                const float2* src = p.src + i * p.inW;
                const __half2* src16 = reinterpret_cast<const __half2*>(p.src) + i * p.inW;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t j = c0 + 32 * u;
                    v[a][u] = (l0 + a < nl && j < p.inW) ? (p.src_c32 ? ld_sample(src16 + j) : __ldg(src + j))
                                                         : make_float2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float2 rot = make_float2(__shfl_sync(0xffffffffu, rot_l.x, l0 + a),
                                               __shfl_sync(0xffffffffu, rot_l.y, l0 + a));
                if (l0 + a >= nl) break;
                float2* dst = p.dst + (i0 + l0 + a) * p.inW;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t j = c0 + 32 * u;
                    if (j < p.inW) dst[j] = cmul(v[a][u], rot);
                }
            }
        }
    }
}

// Carriers that vary along lines: one phase per sample.
__global__ void __launch_bounds__(256) deramp_kernel(const __grid_constant__ DerampParams p) {
    for (int64_t i = blockIdx.y; i < p.inL; i += gridDim.y) {
        const float2* src = p.src + i * p.inW;
        const __half2* src16 = reinterpret_cast<const __half2*>(p.src) + i * p.inW;
        float2* dst = p.dst + i * p.inW;
        const int64_t j0 = (int64_t)blockIdx.x * blockDim.x * 4 + threadIdx.x;
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {     // loads first: four samples in flight per thread
            const int64_t j = j0 + (int64_t)u * blockDim.x;
            v[u] = j < p.inW ? (p.src_c32 ? ld_sample(src16 + j) : __ldg(src + j)) : make_float2(0.f, 0.f);
        }
        const double az = dadd(p.rg_t0, ddiv((double)(i + p.az_first), p.rg_prf));
        const CarrierLine lr = carrier_line(p.rg_car, az), la = carrier_line(p.az_car, az);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t j = j0 + (int64_t)u * blockDim.x;
            if (j >= p.inW) break;
            const double rg = dadd(p.rg_r0, dmul((double)(j + p.rg_first), p.rg_dr));
            const float phase = (float)dadd(carrier_at(p.rg_car, lr, az, rg), carrier_at(p.az_car, la, az, rg));
            float sn, cs;
            sincosf(phase, &sn, &cs);
            dst[j] = cmul(v[u], make_float2(cs, -sn));
        }
    }
}

// FP64 FMA throughput probe: 8 independent dependent chains per thread.
__global__ void __launch_bounds__(256) dfma_probe_kernel(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---- sample codecs (HBM-bound byte work) -----------------------------------
// complex64 -> complex32 (isce3/core/types.py:38-42 to_complex32: numpy's
// float32 -> float16 rounding), complex32 -> complex64 (types.py:45-72,
// exact), and truncate_mantissa (types.py:116-165: AND with a mask keeping
// sign, exponent and the leading mantissa bits).  Grid-stride loops, four
// samples in flight per thread, coalesced 8-byte (and 4-byte) accesses.
__global__ void __launch_bounds__(256) c64_to_c32_kernel(const float2* __restrict__ src, unsigned int* __restrict__ dst,
                                                         int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            v[u] = i < n ? __ldg(src + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) dst[i] = (unsigned int)f32_to_f16_bits(v[u].x) | ((unsigned int)f32_to_f16_bits(v[u].y) << 16);
        }
    }
}

// float16 -> float32 bits as numpy's astype(float32): exact, and a NaN keeps
// its sign and its mantissa bits shifted into the top of the float32 mantissa
__device__ __forceinline__ float f16_bits_to_f32(unsigned short h) {
    if ((h & 0x7c00u) == 0x7c00u && (h & 0x3ffu))
        return __uint_as_float(((unsigned int)(h & 0x8000u) << 16) | 0x7f800000u | ((unsigned int)(h & 0x3ffu) << 13));
    return __half2float(__ushort_as_half(h));
}

__global__ void __launch_bounds__(256) c32_to_c64_kernel(const unsigned int* __restrict__ src,
                                                         float2* __restrict__ dst, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) {
                const unsigned int w = __ldg(src + i);
                v[u] = make_float2(f16_bits_to_f32((unsigned short)(w & 0xffffu)), f16_bits_to_f32((unsigned short)(w >> 16)));
            } else {
                v[u] = make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) dst[i] = v[u];
        }
    }
}

template <typename W>
__global__ void __launch_bounds__(256) mask_words_kernel(W* __restrict__ data, int64_t n, W mask) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
        W v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            v[u] = i < n ? data[i] : W(0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t i = i0 + u * stride;
            if (i < n) data[i] = v[u] & mask;
        }
    }
}

// every element of p set to v (the invalid fill of the raster mode's phase
// outputs); grid-stride, coalesced 8-byte stores
// A request's completion word (mapped host memory): written once the
// kernels before it on the stream have finished, after a system-wide fence
// that orders their outputs before the word.
__global__ void set_flag_kernel(unsigned int* flag) {
    __threadfence_system();
    *(volatile unsigned int*)flag = 1u;
}

__global__ void __launch_bounds__(256) fill_f64_kernel(double* __restrict__ p, int64_t n, double v) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

#endif  // GSLC_PERSISTENT_TU

}  // namespace

#ifndef GSLC_PERSISTENT_TU
cudaError_t probe_fp64(double* out, int blocks, int iters, cudaStream_t s) {
    dfma_probe_kernel<<<blocks, 256, 0, s>>>(out, iters, 0.9999999, 1e-7);
    return cudaGetLastError();
}

template <int PPT>
void launch_geocode_ppt(const GeoParams& p, bool ff, cudaStream_t s) {
    const dim3 block(GBX, GBY);
    const dim3 grid((p.gw + GBX - 1) / GBX, (p.gl + GBY * PPT - 1) / (GBY * PPT));
    if (p.raster) {
        if (p.geo_is_lonlat) {
            if (ff) geocode_kernel<true, true, true, PPT><<<grid, block, 0, s>>>(p);
            else geocode_kernel<true, false, true, PPT><<<grid, block, 0, s>>>(p);
        } else {
            if (ff) geocode_kernel<false, true, true, PPT><<<grid, block, 0, s>>>(p);
            else geocode_kernel<false, false, true, PPT><<<grid, block, 0, s>>>(p);
        }
    } else if (p.geo_is_lonlat) {
        if (ff) geocode_kernel<true, true, false, PPT><<<grid, block, 0, s>>>(p);
        else geocode_kernel<true, false, false, PPT><<<grid, block, 0, s>>>(p);
    } else {
        if (ff) geocode_kernel<false, true, false, PPT><<<grid, block, 0, s>>>(p);
        else geocode_kernel<false, false, false, PPT><<<grid, block, 0, s>>>(p);
    }
}

cudaError_t launch_geocode(const GeoParams& p, int precision, cudaStream_t s, int64_t* launches) {
    // the float-float path covers zero image-grid Doppler with the first
    // iterate at sensingMid; anything else runs in FP64
    const bool ff = precision == 1 && ff_eligible(p);
    launch_geocode_ppt<4>(p, ff, s);     // the plain form uses 32 x 32-pixel tiles
    if (launches) ++*launches;
    return cudaGetLastError();
}

// grid for the codec kernels: a multiple of the SM count, enough for 4
// samples per thread per pass
static unsigned codec_grid(int64_t n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const int64_t want = (n + 1023) / 1024;
    const int64_t cap = (int64_t)sms * 8;
    return (unsigned)std::max<int64_t>(1, std::min(want, cap));
}

cudaError_t launch_codec(int op, const void* src, void* dst, int64_t n, int bits, int word_bytes, cudaStream_t s,
                         int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    const unsigned g = codec_grid(n);
    if (op == 0) {
        c64_to_c32_kernel<<<g, 256, 0, s>>>((const float2*)src, (unsigned int*)dst, n);
    } else if (op == 1) {
        c32_to_c64_kernel<<<g, 256, 0, s>>>((const unsigned int*)src, (float2*)dst, n);
    } else if (word_bytes == 2) {
        const unsigned short m = (unsigned short)(0xffffu << (10 - bits));
        mask_words_kernel<unsigned short><<<g, 256, 0, s>>>((unsigned short*)dst, n, m);
    } else if (word_bytes == 4) {
        const unsigned int m = 0xffffffffu << (23 - bits);
        mask_words_kernel<unsigned int><<<g, 256, 0, s>>>((unsigned int*)dst, n, m);
    } else {
        const unsigned long long m = ~0ull << (52 - bits);
        mask_words_kernel<unsigned long long><<<g, 256, 0, s>>>((unsigned long long*)dst, n, m);
    }
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_set_flag(unsigned int* flag, cudaStream_t s, int64_t* launches) {
    set_flag_kernel<<<1, 1, 0, s>>>(flag);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_fill_f64(double* p, int64_t n, double v, cudaStream_t s, int64_t* launches) {
    if (n <= 0) return cudaSuccess;
    fill_f64_kernel<<<codec_grid(n), 256, 0, s>>>(p, n, v);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_deramp(const DerampParams& p, cudaStream_t s, int64_t* launches) {
    const int64_t chunks = (p.inW + 1023) / 1024;
    if (carrier_line_constant(p.rg_car) && carrier_line_constant(p.az_car)) {
        const int64_t tiles = (p.inL + DR_LINES - 1) / DR_LINES;
        if (chunks < 1 || tiles < 1) return cudaSuccess;
        deramp_lines_kernel<<<dim3((unsigned)chunks, (unsigned)(tiles < 65535 ? tiles : 65535)), 256, 0, s>>>(p);
        if (launches) ++*launches;
        return cudaGetLastError();
    }
    const int64_t lines = p.inL < 65535 ? p.inL : 65535;
    if (chunks < 1 || lines < 1) return cudaSuccess;
    deramp_kernel<<<dim3((unsigned)chunks, (unsigned)lines), 256, 0, s>>>(p);
    if (launches) ++*launches;
    return cudaGetLastError();
}

#else
template <int PPT>
void launch_persistent_ppt(const BatchQueue& q, bool lonlat, bool ff, int blocks, cudaStream_t s) {
    const dim3 block(GBX, GBY);
    if (lonlat) {
        if (ff) geocode_persistent<true, true, PPT><<<blocks, block, 0, s>>>(q);
        else geocode_persistent<true, false, PPT><<<blocks, block, 0, s>>>(q);
    } else {
        if (ff) geocode_persistent<false, true, PPT><<<blocks, block, 0, s>>>(q);
        else geocode_persistent<false, false, PPT><<<blocks, block, 0, s>>>(q);
    }
}

cudaError_t launch_geocode_persistent(const BatchQueue& q, bool lonlat, bool ff, int blocks, cudaStream_t s,
                                      int64_t* launches) {
    switch (q.ppt) {
        case 1: launch_persistent_ppt<1>(q, lonlat, ff, blocks, s); break;
        case 2: launch_persistent_ppt<2>(q, lonlat, ff, blocks, s); break;
        default: launch_persistent_ppt<4>(q, lonlat, ff, blocks, s); break;
    }
    if (launches) ++*launches;
    return cudaGetLastError();
}

template <int PPT>
const void* persistent_fn(bool lonlat, bool ff) {
    return lonlat ? (ff ? (const void*)geocode_persistent<true, true, PPT> : (const void*)geocode_persistent<true, false, PPT>)
                  : (ff ? (const void*)geocode_persistent<false, true, PPT> : (const void*)geocode_persistent<false, false, PPT>);
}

int persistent_blocks_per_sm(bool lonlat, bool ff, int ppt) {
    int n = 0;
    const void* f = ppt == 1 ? persistent_fn<1>(lonlat, ff) : ppt == 2 ? persistent_fn<2>(lonlat, ff) : persistent_fn<4>(lonlat, ff);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, GBX * GBY, 0);
    return n;
}

#endif  // GSLC_PERSISTENT_TU

}  // namespace gslc
