// Block planning on the device: the radar bounding boxes of many geogrid
// blocks in one launch (geometry/boundingbox.cpp:434-641, as
// python/packages/isce3/core/rdr_geo_block_generator.py:7-117 calls it once
// per block), and the DEM statistics that give its heights
// (geometry/DEMInterpolator.cpp:515-560).
//
// A block needs 8 geo2rdr solves (4 corners x {min, max} height), each with
// its own corner-expansion retries.  One thread runs one (corner, height)
// sequence; the 8 threads of a block are 8 consecutive lanes, so the floor /
// ceil min-max and the convergence bookkeeping are warp shuffles.
#include <cuda_runtime.h>

#include "gslc_kernels.cuh"

namespace gslc {
namespace {

// geometry/detail/Geo2Rdr.icc:50-112 (updateAztime): 15-point coarse search
// over the orbit span for the closest approach.
__device__ bool coarse_aztime(const Orbit& o, int look_side, V3 xyz, double& t) {
    constexpr int num = 15;
    const double tstart = o.t0, tend = o.t_end;
    const double dt = (tend - tstart) / (num - 1);
    double r_closest = 1e16, t_closest = -1000.;
    for (int k = 0; k < num; ++k) {
        const double tt = tstart + k * dt;
        if (tt < tstart || tt > tend) continue;
        V3 pos, vel;
        orbit_eval(o, tt, pos, vel);
        const V3 rvec = vsub(xyz, pos);
        if (k == 0 && ((look_side == -1) != (vdot(vcross(rvec, vel), pos) > 0.))) return false;
        const double r = vnorm(rvec);
        if (r < r_closest) { r_closest = r; t_closest = tt; }
    }
    t = (t_closest < 0.) ? 0.5 * (tstart + tend) : t_closest;
    return true;
}

// geometry/geometry.cpp:241-251 over geometry/detail/Geo2Rdr.icc:114-179,
// with a LUT2d Doppler: t is the initial guess on entry (used when inside the
// orbit span) and the last iterate on return, converged or not, so that a
// retry starts where the reference's does.  An iterate outside the span ends
// the solve (the reference's FillNaN orbit makes every later step NaN).
__device__ bool geo2rdr_lut(const Orbit& o, const Lut& dop, int look_side, double wvl, double thr, int maxiter,
                            double dr, V3 xyz, double& t, double& R) {
    if (!(t >= o.t0 && t <= o.t_end) && !coarse_aztime(o, look_side, xyz, t)) return false;
    const double half_wvl = 0.5 * wvl;
    double dt = 0.0;
    for (int i = 0; i < maxiter; ++i) {
        t -= dt;
        if (!(t >= o.t0 && t <= o.t_end)) return false;
        V3 pos, vel;
        orbit_eval(o, t, pos, vel);
        const V3 rvec = vsub(xyz, pos);
        R = vnorm(rvec);
        if (i == 0 && ((look_side == -1) != (vdot(vcross(rvec, vel), pos) > 0.))) return false;
        if (dop.have_data && dop.bounds_error && !(lut_contains(dop, t, R) && lut_contains(dop, t, R + dr)))
            return false;
        const double dopfact = vdot(rvec, vel);
        const double fdop = half_wvl * lut_eval(dop, t, R);
        const double fdopder = (half_wvl * lut_eval(dop, t, R + dr) - fdop) / dr;
        const double fn = dopfact - fdop * R;
        const double c1 = -vdot(vel, vel);
        const double c2 = (fdop / R) + fdopder;
        dt = fn / (c1 + c2 * dopfact);
        if (fabs(dt) < thr) return true;
    }
    return false;
}

__device__ __forceinline__ bool plan_geo2rdr(const PlanParams& p, V3 xyz, double& t, double& R) {
    return geo2rdr_lut(p.orbit, p.dop, p.look_side, p.wvl, p.thr, p.maxiter, p.delta_range, xyz, t, R);
}

__device__ __forceinline__ int shfl_min8(int v) {
#pragma unroll
    for (int m = 1; m < 8; m <<= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, m));
    return v;
}
__device__ __forceinline__ int shfl_max8(int v) {
#pragma unroll
    for (int m = 1; m < 8; m <<= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, m));
    return v;
}
__device__ __forceinline__ int shfl_or8(int v) {
#pragma unroll
    for (int m = 1; m < 8; m <<= 1) v |= __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

// float -> int as std::floor / std::ceil then static_cast<int>, saturated
// where the reference's cast would be undefined
__device__ __forceinline__ int to_int(double v) { return (int)fmax(fmin(v, 2147483647.0), -2147483648.0); }

// Lane l of a group of 8: corner (line, pixel) = ((l >> 2) & 1, (l >> 1) & 1),
// height index l & 1.  Corner order and expansion directions follow
// boundingbox.cpp:473-493: top-left (-1, -1), top-right (+1, -1),
// bottom-left (-1, +1), bottom-right (+1, +1) in (x, y) geogrid steps.
__global__ void __launch_bounds__(256) radar_bbox_kernel(const __grid_constant__ PlanParams p) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int blk = gid >> 3, lane = gid & 7;
    const int line = (lane >> 2) & 1, pixel = (lane >> 1) & 1, ih = lane & 1;
    const bool active = blk < p.n_blocks;
    int conv = 0, projfail = 0;
    int fa = 0x7fffffff, la = (int)0x80000000, fr = 0x7fffffff, lr = (int)0x80000000;
    if (active) {
        const double* b = p.blocks + (int64_t)blk * 6;   // start x, y, spacing x, y, width, length
        const double sx = b[2], sy = b[3];
        // corner (boundingbox.cpp:499-506): start + spacing * {0,1} * size
        const double y0 = dadd(b[1], dmul(dmul(sy, (double)line), b[5]));
        const double x0 = dadd(b[0], dmul(dmul(sx, (double)pixel), b[4]));
        const int exd = pixel ? 1 : -1, eyd = line ? 1 : -1;
        const double h = (double)(ih ? p.hmax : p.hmin);
        double t = p.t_mid, R = p.r0;
        bool ok = false;
        for (int it = 0; !ok && it < p.expansion; ++it) {
            const double x = dadd(x0, dmul((double)(it * exd), sx));
            const double y = dadd(y0, dmul((double)(it * eyd), sy));
            double lon, lat;
            if (p.geo_is_lonlat) {
                lon = ddiv(dmul(x, PI), 180.0);     // LonLat::inverse (Projections.h:136-140)
                lat = ddiv(dmul(y, PI), 180.0);
            } else if (!utm_inverse(p.utm, x, y, lon, lat)) {
                projfail = 1;
                break;
            }
            double slon, clon, slat, clat;
            sincos(lon, &slon, &clon);
            sincos(lat, &slat, &clat);
            const V3 xyz = lonlat_to_xyz_sc(p.ell_a, p.ell_e2, slon, clon, slat, clat, h);
            ok = plan_geo2rdr(p, xyz, t, R);
        }
        if (ok && !projfail) {
            conv = 1;
            const double az = (t - p.t0) * p.prf;
            const double rg = (R - p.r0) / p.dr;
            fa = to_int(floor(az));
            la = to_int(ceil(az));
            fr = to_int(floor(rg));
            lr = to_int(ceil(rg));
        }
    }
    fa = shfl_min8(fa);
    la = shfl_max8(la);
    fr = shfl_min8(fr);
    lr = shfl_max8(lr);
    projfail = shfl_or8(projfail);
    // corner k converged with either height: bit k
    int cbits = shfl_or8(conv ? 1 << (lane >> 1) : 0);
    if (!active || lane != 0) return;
    int32_t* out = p.out + (int64_t)blk * 6;
    // initial values of boundingbox.cpp:465-470
    const int max_az = (int)(p.length - 1), max_rg = (int)(p.width - 1);
    fa = min(fa, max_az);
    la = max(la, 0);
    fr = min(fr, max_rg);
    lr = max(lr, 0);
    out[0] = fa; out[1] = la; out[2] = fr; out[3] = lr;
    if (projfail) { out[4] = 3; out[5] = 0; return; }
    if (cbits != 0xf) { out[4] = 1; out[5] = ~cbits & 0xf; return; }
    int why = 0;
    if (fa <= 0 && la <= 0) why |= 1;
    if (fa >= max_az && la >= max_az) why |= 2;
    if (fr <= 0 && lr <= 0) why |= 4;
    if (fr >= max_rg && lr >= max_rg) why |= 8;
    if (why) { out[4] = 2; out[5] = why; return; }
    out[0] = max(fa - p.margin, 0);
    out[2] = max(fr - p.margin, 0);
    out[1] = min(la + p.margin, max_az);
    out[3] = min(lr + p.margin, max_rg);
    out[4] = 0;
    out[5] = 0;
}

// ---- radar grid metadata cubes (geometry/metadataCubes.cpp:276-489) --------
// One thread per (height, line, column) point: geo2rdr with the grid Doppler
// (slant range, azimuth time), then with the native Doppler for the platform
// state, and the vectors of writeVectorDerivedCubes (:74-274).  The reference
// starts each point's solves from the previous point's results (a chain
// through each height layer); one launch here is one pass that solves every
// point from the starts the host derived from the previous pass, and writes
// every output (NaN where a solve failed), the final iterates and the
// statuses for the next derivation.
__device__ __forceinline__ V3 vunit(V3 v) {
    const double n = vnorm(v);
    return {v.x / n, v.y / n, v.z / n};
}

// core/DenseMatrix.h:73-79 (xyzToEnu) applied to v
__device__ __forceinline__ V3 to_enu(double slat, double clat, double slon, double clon, V3 v) {
    return {-slon * v.x + clon * v.y, -slat * clon * v.x - slat * slon * v.y + clat * v.z,
            clat * clon * v.x + clat * slon * v.y + slat * v.z};
}

// core/Ellipsoid.h:197-231 (Vermeille 2002): latitude and longitude of an
// ECEF point (the height is not needed here)
__device__ void xyz_to_latlon(double a, double e2, V3 x, double& lat, double& lon) {
    const double e4 = e2 * e2, a2 = a * a;
    const double p = (x.x * x.x + x.y * x.y) / a2;
    const double q = ((1. - e2) * (x.z * x.z)) / a2;
    const double r = (p + q - e4) / 6.;
    const double s = (e4 * p * q) / (4. * (r * r * r));
    const double t = pow(1. + s + sqrt(s * (2. + s)), 1. / 3.);
    const double u = r * (1. + t + (1. / t));
    const double rv = sqrt(u * u + (e4 * q));
    const double w = (e2 * (u + rv - q)) / (2. * rv);
    const double k = sqrt(u + rv + w * w) - w;
    const double d = (k * sqrt(x.x * x.x + x.y * x.y)) / (k + e2);
    lat = atan2(x.z, d);
    lon = atan2(x.y, x.x);
}

__global__ void __launch_bounds__(256) radar_grid_cubes_kernel(const __grid_constant__ CubeParams p) {
    const int64_t plane = (int64_t)p.length * p.width;
    const int64_t n = plane * p.n_heights;
    const double dnan = __longlong_as_double(0x7ff8000000000000LL);
    const float fnan = __int_as_float(0x7fc00000);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int hc = (int)(k / plane);
        const int64_t r = k - hc * plane;
        const int i = (int)(r / p.width), j = (int)(r - (int64_t)i * p.width);
        const double h = p.heights[hc];
        double sr = dnan, at = dnan, gv = dnan;
        float inc = fnan, lx = fnan, ly = fnan, ax = fnan, ay = fnan, el = fnan;
        unsigned char st = 0;
        double t = p.start_grid[k], tn = p.start_native[k];
        // pixel centre (metadataCubes.cpp:341-345), reference rounding
        const double y = dadd(p.gy0, dmul(0.5 + (double)i, p.gdy));
        const double x = dadd(p.gx0, dmul(0.5 + (double)j, p.gdx));
        double lon, lat;
        bool proj_ok = true;
        if (p.geo_is_lonlat) {
            lon = ddiv(dmul(x, PI), 180.0);
            lat = ddiv(dmul(y, PI), 180.0);
        } else if (!utm_inverse(p.utm, x, y, lon, lat)) {
            atomicOr(p.err, 1);
            proj_ok = false;
        }
        if (proj_ok) {
            double slon, clon, slat, clat;
            sincos(lon, &slon, &clon);
            sincos(lat, &slat, &clat);
            const V3 target = lonlat_to_xyz_sc(WGS84_A, WGS84_E2, slon, clon, slat, clat, h);
            double R = p.mid_range;
            if (geo2rdr_lut(p.orbit, p.grid_dop, p.look_side, p.wvl, p.thr, p.maxiter, p.delta_range, target, t, R)) {
                st = 1;
                sr = R;
                at = t;
                double Rn = p.mid_range;
                if (p.want_vectors && geo2rdr_lut(p.orbit, p.nat_dop, p.look_side, p.wvl, p.thr, p.maxiter,
                                                  p.delta_range, target, tn, Rn)) {
                    st |= 2;
                    V3 sat, vel;
                    orbit_eval(p.orbit, tn, sat, vel);
                    // law of cosines (metadataCubes.cpp:118-132)
                    const double slant = vnorm(vsub(target, sat));
                    const double rt = vnorm(target), rp = vnorm(sat);
                    const double cos_alpha = ((rt * rt + rp * rp - slant * slant) / (2 * rt * rp));
                    gv = cos_alpha * rt * vnorm(vel) / rp;
                    const V3 look = vunit(vsub(sat, target));
                    if (p.elevation) {
                        double sl, so, ss, cs, sso, cso;
                        xyz_to_latlon(WGS84_A, WGS84_E2, sat, sl, so);
                        sincos(sl, &ss, &cs);
                        sincos(so, &sso, &cso);
                        const V3 les = vunit(to_enu(ss, cs, sso, cso, look));
                        el = (float)(acos(les.z) * 180.0 / PI);
                    }
                    const V3 le = vunit(to_enu(slat, clat, slon, clon, look));
                    inc = (float)(acos(fabs(le.z)) * 180.0 / PI);
                    lx = (float)le.x;
                    ly = (float)le.y;
                    const V3 atv = vunit(to_enu(slat, clat, slon, clon, vel));
                    ax = (float)atv.x;
                    ay = (float)atv.y;
                }
            }
        }
        p.t_grid[k] = t;
        p.t_native[k] = tn;
        p.status[k] = st;
        if (p.slant_range) p.slant_range[k] = sr;
        if (p.azimuth_time) p.azimuth_time[k] = at;
        if (p.incidence) p.incidence[k] = inc;
        if (p.los_x) p.los_x[k] = lx;
        if (p.los_y) p.los_y[k] = ly;
        if (p.along_x) p.along_x[k] = ax;
        if (p.along_y) p.along_y[k] = ay;
        if (p.elevation) p.elevation[k] = el;
        if (p.ground_velocity) p.ground_velocity[k] = gv;
    }
}

// DEM statistics, pass 1: per-block min, max, sum and NaN count over a
// strided float raster (coalesced along rows, grid-stride over lines).
// Starting values are the reference's +-FLT_MAX.
using DemPartial = DemStats;
constexpr float FMAXV = 3.402823466e+38f;

__global__ void __launch_bounds__(256) dem_stats_partial(const float* __restrict__ z, int64_t length, int64_t width,
                                                         int64_t stride, DemPartial* __restrict__ part) {
    float mn = FMAXV, mx = -FMAXV;
    double sum = 0.0;
    long long nan = 0;
    const int64_t n = length * width;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / width, c = i - r * width;
        const float v = __ldg(z + r * stride + c);
        if (isnan(v)) { ++nan; continue; }
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        sum += (double)v;
    }
    __shared__ DemPartial s[256];
    s[threadIdx.x] = {mn, mx, sum, nan};
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            DemPartial a = s[threadIdx.x], b = s[threadIdx.x + w];
            s[threadIdx.x] = {fminf(a.mn, b.mn), fmaxf(a.mx, b.mx), a.sum + b.sum, a.nan + b.nan};
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// pass 2: one block folds the partials in a fixed order (deterministic)
__global__ void __launch_bounds__(256) dem_stats_final(const DemPartial* __restrict__ part, int n, DemPartial* out) {
    __shared__ DemPartial s[256];
    DemPartial a{FMAXV, -FMAXV, 0.0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const DemPartial b = part[i];
        a = {fminf(a.mn, b.mn), fmaxf(a.mx, b.mx), a.sum + b.sum, a.nan + b.nan};
    }
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            DemPartial x = s[threadIdx.x], y = s[threadIdx.x + w];
            s[threadIdx.x] = {fminf(x.mn, y.mn), fmaxf(x.mx, y.mx), x.sum + y.sum, x.nan + y.nan};
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

}  // namespace

cudaError_t launch_radar_bbox(const PlanParams& p, cudaStream_t s, int64_t* launches) {
    if (p.n_blocks <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t n = (int64_t)p.n_blocks * 8;
    radar_bbox_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(p);
    if (launches) ++*launches;
    return cudaGetLastError();
}

cudaError_t launch_radar_grid_cubes(const CubeParams& p, cudaStream_t s, int64_t* launches) {
    const int64_t n = (int64_t)p.length * p.width * p.n_heights;
    if (n <= 0) return cudaSuccess;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + 255) / 256;
    const unsigned grid = (unsigned)(want < (int64_t)sms * 8 ? want : (int64_t)sms * 8);
    radar_grid_cubes_kernel<<<grid, 256, 0, s>>>(p);
    if (launches) ++*launches;
    return cudaGetLastError();
}

size_t dem_stats_scratch_bytes() { return (size_t)(DEM_STATS_BLOCKS + 1) * sizeof(DemPartial); }

cudaError_t launch_dem_stats(const float* z, int64_t length, int64_t width, int64_t stride, void* scratch,
                             DemStats* host_out, cudaStream_t s, int64_t* launches) {
    DemPartial* part = reinterpret_cast<DemPartial*>(scratch);
    DemPartial* fin = part + DEM_STATS_BLOCKS;
    dem_stats_partial<<<DEM_STATS_BLOCKS, 256, 0, s>>>(z, length, width, stride, part);
    dem_stats_final<<<1, 256, 0, s>>>(part, DEM_STATS_BLOCKS, fin);
    if (launches) *launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(host_out, fin, sizeof(DemPartial), cudaMemcpyDeviceToHost, s);
}

}  // namespace gslc
