// Raster interpolation of the CUDA raster geocoder for every data type and
// method it accepts (cxx/isce3/cuda/geocode/Geocode.cu:203-287 with the
// device interpolators of cxx/isce3/cuda/core/: gpuNearestNeighbor,
// gpuBilinear, gpuBicubic, gpuSpline2d order 6, gpuSinc2d).  The radar
// coordinates of each geogrid pixel come from the fused kernel's coordinate
// pass (NaN where masked); here one thread per geogrid pixel interpolates one
// raster.  The SINC complex64 case stays fused in geocode_kernel.
//
// Complex rasters: in the reference every complex operand that meets a
// weight is real ((w, 0), or a real p of the spline), so its thrust complex
// arithmetic equals the same real arithmetic on each component; one
// real-valued interpolator per component type (float, double) covers all
// four floating types.  Arithmetic uses round-to-nearest intrinsics (no FMA
// contraction), with the reference's mixed float/double promotions.
#include <cuda_runtime.h>
#include <math_constants.h>

#include "gslc_kernels.cuh"

namespace gslc {
namespace {

template <typename S> __device__ __forceinline__ S radd(S a, S b);
template <typename S> __device__ __forceinline__ S rsub(S a, S b);
template <typename S> __device__ __forceinline__ S rmul(S a, S b);
template <typename S> __device__ __forceinline__ S rdiv(S a, S b);
template <> __device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// Component c (0 or 1) of sample (row, col) of a raster of NC-component samples.
template <typename S, int NC>
struct View {
    const S* z;
    int64_t nx;
    int c;
    __device__ __forceinline__ S operator()(int64_t row, int64_t col) const { return z[(row * nx + col) * NC + c]; }
};

// gpuNearestNeighborInterpolator.cu:8-15
template <typename S, int NC>
__device__ S interp_nearest(double x, double y, const View<S, NC>& z) {
    return z((int64_t)round(y), (int64_t)round(x));
}

// gpuBilinearInterpolator.cu:78-108: weights formed in double, cast to the
// sample type; the divisions by (x2 - x1)(y2 - y1) = 1 are exact and kept.
template <typename S, int NC>
__device__ S interp_bilinear(double x, double y, const View<S, NC>& z) {
    const int64_t x1 = (int64_t)floor(x), x2 = (int64_t)ceil(x);
    const int64_t y1 = (int64_t)floor(y), y2 = (int64_t)ceil(y);
    const S q11 = z(y1, x1), q12 = z(y2, x1), q21 = z(y1, x2), q22 = z(y2, x2);
    const double dx2 = __dsub_rn((double)x2, x), dx1 = __dsub_rn(x, (double)x1);
    const double dy2 = __dsub_rn((double)y2, y), dy1 = __dsub_rn(y, (double)y1);
    const double ex = (double)(x2 - x1), ey = (double)(y2 - y1);
    if (y1 == y2 && x1 == x2) return q11;
    if (y1 == y2)
        return radd(rmul((S)__ddiv_rn(dx2, ex), q11), rmul((S)__ddiv_rn(dx1, ex), q21));
    if (x1 == x2)
        return radd(rmul((S)__ddiv_rn(dy2, ey), q11), rmul((S)__ddiv_rn(dy1, ey), q12));
    const S den = (S)__dmul_rn(ex, ey);
    S r = rdiv(rmul(q11, (S)__dmul_rn(dx2, dy2)), den);
    r = radd(r, rdiv(rmul(q21, (S)__dmul_rn(dx1, dy2)), den));
    r = radd(r, rdiv(rmul(q12, (S)__dmul_rn(dx2, dy1)), den));
    return radd(r, rdiv(rmul(q22, (S)__dmul_rn(dx1, dy1)), den));
}

// The bicubic weight matrix of gpuBicubicInterpolator.cu (16 x 16, row i
// gives coefficient c_i from the 16 corner values and derivatives).
__constant__ signed char c_bicubic_w[256] = {
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

// gpuBicubicInterpolator.cu:104-188 in the sample type, the reference's
// sample offsets kept as they are (including its y-derivative stencils at
// the x2 and right-hand corners).
template <typename S, int NC>
__device__ S interp_bicubic(double x, double y, const View<S, NC>& z) {
    const int64_t x1 = (int64_t)floor(x), x2 = (int64_t)ceil(x);
    const int64_t y1 = (int64_t)floor(y), y2 = (int64_t)ceil(y);
    const S denom = (S)2.0, scale = (S)0.25;
    S q[16];
    q[0] = z(y1, x1); q[1] = z(y1, x2); q[2] = z(y2, x2); q[3] = z(y2, x1);
    q[4] = rdiv(rsub(z(y1, x1 + 1), z(y1, x1 - 1)), denom);
    q[5] = rdiv(rsub(z(y1, x2 + 1), z(y1, x2 - 1)), denom);
    q[6] = rdiv(rsub(z(y2, x2 + 1), z(y2, x2 - 1)), denom);
    q[7] = rdiv(rsub(z(y2, x1 + 1), z(y2, x1 - 1)), denom);
    q[8] = rdiv(rsub(z(y1 + 1, x1), z(y1 - 1, x1)), denom);
    q[9] = rdiv(rsub(z(y1 + 1, x2 + 1), z(y1 - 1, x2)), denom);
    q[10] = rdiv(rsub(z(y2 + 1, x2 + 1), z(y2 - 1, x2)), denom);
    q[11] = rdiv(rsub(z(y2 + 1, x1 + 1), z(y2 - 1, x1)), denom);
    const int64_t xs[4] = {x1, x2, x2, x1}, ys[4] = {y1, y1, y2, y2};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int64_t xx = xs[k], yy = ys[k];
        S d = rsub(z(yy + 1, xx + 1), z(yy - 1, xx + 1));
        d = rsub(d, z(yy + 1, xx - 1));
        d = radd(d, z(yy - 1, xx - 1));
        q[12 + k] = rmul(scale, d);
    }
    S c[16];
#pragma unroll 1
    for (int i = 0; i < 16; ++i) {
        S qq = (S)0.0;
        for (int j = 0; j < 16; ++j) qq = radd(qq, rmul((S)c_bicubic_w[i * 16 + j], q[j]));
        c[i] = qq;
    }
    const S t = (S)__dsub_rn(x, (double)x1), u = (S)__dsub_rn(y, (double)y1);
    S ret = (S)0.0;
    for (int i = 3; i >= 0; --i) {
        // t * ret + ((c3 u + c2) u + c1) u + c0, added left to right
        S v = radd(rmul(c[i * 4 + 3], u), c[i * 4 + 2]);
        v = rmul(radd(rmul(v, u), c[i * 4 + 1]), u);
        ret = radd(radd(rmul(t, ret), v), c[i * 4]);
    }
    return ret;
}

// gpuSpline2dInterpolator.cu (_initSpline, _spline, interpolate; order 6):
// samples and the R, Q arrays in the sample type S, the terms with double
// literals (p, 0.5 R, R / 6.0, ...) in double, as C++ promotes them.
template <typename S>
__device__ void spline_init(const S* Y, S* R, S* Q) {
    Q[0] = (S)0.0;
    R[0] = (S)0.0;
    for (int i = 1; i < 5; ++i) {
        const double p = __ddiv_rn(1.0, __dadd_rn(__dmul_rn(0.5, (double)Q[i - 1]), 2.0));
        Q[i] = (S)__dmul_rn(-0.5, p);
        S t = radd(rsub(Y[i + 1], rmul((S)2, Y[i])), Y[i - 1]);
        t = rmul((S)3, t);
        R[i] = (S)__dmul_rn(__dsub_rn((double)t, __dmul_rn(0.5, (double)R[i - 1])), p);
    }
    R[5] = (S)0.0;
    for (int i = 4; i > 0; --i) R[i] = radd(rmul(Q[i], R[i + 1]), R[i]);
}

template <typename S>
__device__ S spline_eval(double x, const S* Y, const S* R) {
    constexpr int n = 6;
    if (x < 1.0) {
        const double d = __dsub_rn((double)rsub(Y[1], Y[0]), __ddiv_rn((double)R[1], 6.0));
        return (S)__dadd_rn((double)Y[0], __dmul_rn(__dsub_rn(x, 1.0), d));
    }
    if (x > n) {
        const double d = __dadd_rn((double)rsub(Y[n - 1], Y[n - 2]), __ddiv_rn((double)R[n - 2], 6.0));
        return (S)__dadd_rn((double)Y[n - 1], __dmul_rn(__dsub_rn(x, (double)n), d));
    }
    const int j = (int)floor(x);
    const double xx = __dsub_rn(x, (double)j);
    double t0 = __dsub_rn((double)rsub(Y[j], Y[j - 1]), __ddiv_rn((double)R[j - 1], 3.0));
    t0 = __dsub_rn(t0, __ddiv_rn((double)R[j], 6.0));
    const double inner = __dmul_rn(xx, (double)rdiv(rsub(R[j], R[j - 1]), (S)6));
    const double t1 = __dmul_rn(xx, __dadd_rn(__ddiv_rn((double)R[j - 1], 2.0), inner));
    return (S)__dadd_rn((double)Y[j - 1], __dmul_rn(xx, __dadd_rn(t0, t1)));
}

template <typename S, int NC>
__device__ S interp_biquintic(double x, double y, const View<S, NC>& z, int64_t ny) {
    const int i0 = (int)y - 2, j0 = (int)x - 2;      // order 6 is even: truncation, then - (6/2 - 1)
    S A[6], R[6], Q[6], HC[6];
    for (int i = 0; i < 6; ++i) {
        const int64_t indi = min(max((int64_t)(i0 + i), (int64_t)0), ny - 2);
        for (int j = 0; j < 6; ++j) {
            const int64_t indj = min(max((int64_t)(j0 + j), (int64_t)0), z.nx - 2);
            A[j] = z(indi + 1, indj + 1);
        }
        spline_init(A, R, Q);
        HC[i] = spline_eval(__dsub_rn(x, (double)j0), A, R);
    }
    spline_init(HC, R, Q);
    return spline_eval(__dsub_rn(y, (double)i0), HC, R);
}

// Geocode.cu:243-277 with gpuSinc2dInterpolator.cu:103-140: a 9 x 9 chip
// around (floor y, floor x), Sinc2d at (4 + frac x, 4 + frac y) with the
// table cast to the sample type; terms (chip * ky) * kx summed row by row.
template <typename S, int NC>
__device__ S interp_sinc(double x, double y, const View<S, NC>& z, const S* table) {
    const int xi = __double2int_rd(x), yi = __double2int_rd(y);
    const double X = __dadd_rn(4.0, __dsub_rn(x, (double)xi)), Y = __dadd_rn(4.0, __dsub_rn(y, (double)yi));
    const int ix = __double2int_rd(X), iy = __double2int_rd(Y);
    if (!(ix >= SINC_HALF - 1 && ix <= SINC_ONE - SINC_HALF - 1 && iy >= SINC_HALF - 1 && iy <= SINC_ONE - SINC_HALF - 1))
        return (S)0.0;
    const double fx = __dsub_rn(X, (double)ix), fy = __dsub_rn(Y, (double)iy);
    const int ifx = min(max(0, (int)(fx * SINC_SUB)), SINC_SUB - 1);
    const int ify = min(max(0, (int)(fy * SINC_SUB)), SINC_SUB - 1);
    const int px = ix + SINC_HALF, py = iy + SINC_HALF;
    S acc = (S)0.0;
    for (int i = 0; i < SINC_LEN; ++i) {
        const S ky = table[ify * SINC_LEN + i];
        const int64_t row = yi + (py - i) - SINC_HALF;
        for (int j = 0; j < SINC_LEN; ++j) {
            const S kx = table[ifx * SINC_LEN + j];
            acc = radd(acc, rmul(rmul(z(row, xi + (px - j) - SINC_HALF), ky), kx));
        }
    }
    return acc;
}

// Geocode.cu:232-241: masked pixels (NaN coordinates) and chips that would
// come within 4 samples of the raster's edge take the invalid value.
__device__ __forceinline__ bool raster_inside(const RasterInterpParams& p, double x, double y) {
    return !(isnan(x) || isnan(y) || x < 4.0 || y < 4.0 || x >= (double)p.W - 4.0 || y >= (double)p.L - 4.0);
}

template <typename S, int NC, int METHOD>
__global__ void __launch_bounds__(256) raster_interp_kernel(const __grid_constant__ RasterInterpParams p) {
    const S* src = reinterpret_cast<const S*>(p.rdr);
    S* dst = reinterpret_cast<S*>(p.out);
    const S* table = reinterpret_cast<const S*>(p.sinc);
    const S inv = (S)p.invalid;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += (int64_t)gridDim.x * blockDim.x) {
        const double y = p.az[k], x = p.rg[k];
        const bool ok = raster_inside(p, x, y);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            S v = inv;
            if (ok) {
                const View<S, NC> z{src, p.W, c};
                if (METHOD == 0) v = interp_sinc(x, y, z, table);
                else if (METHOD == 1) v = interp_bilinear(x, y, z);
                else if (METHOD == 2) v = interp_bicubic(x, y, z);
                else if (METHOD == 3) v = interp_nearest(x, y, z);
                else v = interp_biquintic(x, y, z, p.L);
            }
            dst[k * NC + c] = v;
        }
    }
}

// unsigned integer rasters: nearest neighbour only (Geocode.cu:290-302)
template <typename U>
__global__ void __launch_bounds__(256) raster_nearest_uint_kernel(const __grid_constant__ RasterInterpParams p) {
    const U* src = reinterpret_cast<const U*>(p.rdr);
    U* dst = reinterpret_cast<U*>(p.out);
    const U inv = (U)p.invalid;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += (int64_t)gridDim.x * blockDim.x) {
        const double y = p.az[k], x = p.rg[k];
        dst[k] = raster_inside(p, x, y) ? src[(int64_t)round(y) * p.W + (int64_t)round(x)] : inv;
    }
}

template <typename S, int NC>
void launch_typed(const RasterInterpParams& p, unsigned grid, cudaStream_t s) {
    switch (p.method) {
    case 0: raster_interp_kernel<S, NC, 0><<<grid, 256, 0, s>>>(p); break;
    case 1: raster_interp_kernel<S, NC, 1><<<grid, 256, 0, s>>>(p); break;
    case 2: raster_interp_kernel<S, NC, 2><<<grid, 256, 0, s>>>(p); break;
    case 3: raster_interp_kernel<S, NC, 3><<<grid, 256, 0, s>>>(p); break;
    default: raster_interp_kernel<S, NC, 4><<<grid, 256, 0, s>>>(p); break;
    }
}

}  // namespace

cudaError_t launch_raster_interp(const RasterInterpParams& p, cudaStream_t s, int64_t* launches) {
    if (p.n <= 0) return cudaSuccess;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (p.n + 255) / 256;
    const unsigned grid = (unsigned)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
    switch (p.dtype) {
    case RASTER_F32: launch_typed<float, 1>(p, grid, s); break;
    case RASTER_C64: launch_typed<float, 2>(p, grid, s); break;
    case RASTER_F64: launch_typed<double, 1>(p, grid, s); break;
    case RASTER_C128: launch_typed<double, 2>(p, grid, s); break;
    case RASTER_U8: raster_nearest_uint_kernel<uint8_t><<<grid, 256, 0, s>>>(p); break;
    case RASTER_U16: raster_nearest_uint_kernel<uint16_t><<<grid, 256, 0, s>>>(p); break;
    default: raster_nearest_uint_kernel<uint32_t><<<grid, 256, 0, s>>>(p); break;
    }
    if (launches) ++*launches;
    return cudaGetLastError();
}

}  // namespace gslc
