// TEST INFRASTRUCTURE: a C ABI over the reference's own interpolators
// (core/BilinearInterpolator.cpp, BicubicInterpolator.cpp,
// NearestNeighborInterpolator.cpp, Spline2dInterpolator.cpp,
// Sinc2dInterpolator.cpp), LUT2d (core/LUT2d.cpp) and Poly2d
// (core/Poly2d.cpp), built where they lie in the reference checkout by
// oracle/Makefile, target "ref", with ref_shim/ standing in for Eigen 3.3.7
// and pyre-journal).  The oracle's restatements of the same interpolators
// are checked against it bit for bit.  Nothing in the product uses it.
#include <complex>
#include <memory>

#include "isce3/core/Interpolator.h"
#include "isce3/core/LUT2d.h"
#include "isce3/core/Poly2d.h"

using isce3::core::dataInterpMethod;

namespace {
template <typename U>
using MapOf = Eigen::Map<const isce3::core::EArray2D<U>>;
}

extern "C" {

// createInterpolator<double>(method) (core/Interpolator.h: biquintic of
// order 6, sinc of SINC_LEN taps at SINC_SUB phases) at (x, y) of the
// row-major ny x nx table z.  method: isce3 dataInterpMethod.
double ref_interp2d_double(int method, const double* z, int ny, int nx, double x, double y) {
    std::unique_ptr<isce3::core::Interpolator<double>> it(
            isce3::core::createInterpolator<double>(static_cast<dataInterpMethod>(method)));
    return it->interpolate(x, y, MapOf<double>(z, ny, nx));
}

// Spline2dInterpolator<float>(6), the DEM interpolator's spline
// (geometry/DEMInterpolator.cpp), at (x, y) of a row-major float table.
float ref_spline2d_float(const float* z, int ny, int nx, double x, double y) {
    const isce3::core::Spline2dInterpolator<float> it(6);
    return it.interpolate(x, y, MapOf<float>(z, ny, nx));
}

// Sinc2dInterpolator<std::complex<float>>(SINC_LEN, SINC_SUB), the SLC
// interpolator of geocodeSlc.cpp:476-494, at (x, y) of a row-major complex64
// table (interleaved re, im); out: re, im.
void ref_sinc2d_cfloat(const float* z, int ny, int nx, double x, double y, float* out) {
    const isce3::core::Sinc2dInterpolator<std::complex<float>> it(isce3::core::SINC_LEN, isce3::core::SINC_SUB);
    const std::complex<float> v =
            it.interpolate(x, y, MapOf<std::complex<float>>(reinterpret_cast<const std::complex<float>*>(z), ny, nx));
    out[0] = v.real();
    out[1] = v.imag();
}

// LUT2d<double>(xstart, ystart, dx, dy, data, method, bounds_error).eval(y, x)
// (core/LUT2d.cpp:18-27, 124-158) over the row-major ny x nx table z.
double ref_lut2d_eval(double xstart, double ystart, double dx, double dy, const double* z, int ny, int nx, int method,
                      int bounds_error, double y, double x) {
    std::vector<double> copy(z, z + (size_t)ny * nx);
    const isce3::core::Matrix<double> data(copy.data(), ny, nx);
    const isce3::core::LUT2d<double> lut(xstart, ystart, dx, dy, data, static_cast<dataInterpMethod>(method),
                                         bounds_error != 0);
    return lut.eval(y, x);
}

// Poly2d::eval (core/Poly2d.cpp:8-24); coeffs row-major (y_order + 1) x (x_order + 1)
double ref_poly2d_eval(int x_order, int y_order, double x_mean, double y_mean, double x_norm, double y_norm,
                       const double* coeffs, double y, double x) {
    isce3::core::Poly2d p(x_order, y_order, x_mean, y_mean, x_norm, y_norm);
    for (size_t i = 0; i < p.coeffs.size(); ++i) p.coeffs[i] = coeffs[i];
    return p.eval(y, x);
}

}  // extern "C"
