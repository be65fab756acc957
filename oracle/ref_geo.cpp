// The reference's own geometry code, compiled from its sources — TEST
// INFRASTRUCTURE (the oracle's pin; never used by the product).
//
// This file contains no reference code: it includes the reference's headers
// (geometry/detail/Geo2Rdr.icc, core/detail/InterpolateOrbit.icc,
// core/Linspace.icc, core/Ellipsoid.h) and is linked with its
// core/Projections.cpp and except/Error.cpp, all compiled where they lie by
// oracle/Makefile's "ref" target, with oracle/ref_shim standing in for
// Eigen 3.3.7.  It adds a C ABI over them so that tests can compare the
// oracle's restatement with the reference's arithmetic bit for bit.
//
// RefOrbit provides what the templated orbit interpolation and geo2rdr read
// from isce3::core::Orbit (core/Orbit.h:94-205): the uniform time grid as a
// Linspace, state vectors, interpolation method, start/mid/end times, and
// interpolate() forwarding to detail::interpolateOrbit (core/Orbit.cpp:71-86).
// ConstDoppler is a LUT2d without data (core/LUT2d.h:84-95, LUT2d.cpp:124-130:
// contains() is true, eval() returns the reference value).
#include <cstdint>
#include <vector>

#include <isce3/core/Ellipsoid.h>
#include <isce3/core/Linspace.h>
#include <isce3/core/LookSide.h>
#include <isce3/core/Orbit.h>
#include <isce3/core/Projections.h>
#include <isce3/core/detail/InterpolateOrbit.h>
#include <isce3/geometry/detail/Geo2Rdr.h>

// core/DateTime.h:151 defines the header-level constant MIN_DATE_TIME, whose
// constructor lives in core/DateTime.cpp; that file needs pyre-journal, which
// is absent.  Nothing on the geometry path reads the constant, so the
// constructor is defined here as an empty link stub.
isce3::core::DateTime::DateTime(int, int, int) {}

using isce3::core::Linspace;
using isce3::core::OrbitInterpBorderMode;
using isce3::core::OrbitInterpMethod;
using isce3::core::Vec3;

namespace {

struct RefOrbit {
    Linspace<double> t;
    std::vector<Vec3> pos, vel;
    OrbitInterpMethod method;

    RefOrbit(const double* p, const double* v, int n, double first, double spacing, int m)
        : t(first, spacing, n), method(m == 1 ? OrbitInterpMethod::Legendre : OrbitInterpMethod::Hermite) {
        pos.resize(n);
        vel.resize(n);
        for (int i = 0; i < n; ++i) {
            pos[i] = Vec3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
            vel[i] = Vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        }
    }
    OrbitInterpMethod interpMethod() const { return method; }
    double startTime() const { return t[0]; }
    double midTime() const { return startTime() + 0.5 * (size() - 1) * spacing(); }
    double endTime() const { return t[size() - 1]; }
    double spacing() const { return t.spacing(); }
    int size() const { return t.size(); }
    const Linspace<double>& time() const { return t; }
    double time(int i) const { return t[i]; }
    const Vec3& position(int i) const { return pos[i]; }
    const Vec3& velocity(int i) const { return vel[i]; }
    isce3::error::ErrorCode interpolate(Vec3* p, Vec3* v, double tt, OrbitInterpBorderMode m) const {
        return isce3::core::detail::interpolateOrbit(p, v, *this, tt, m);
    }
};

struct ConstDoppler {
    double ref;
    bool bounds;
    bool boundsError() const { return bounds; }
    bool contains(double, double) const { return true; }
    double eval(double, double) const { return ref; }
};

}  // namespace

extern "C" {

// Orbit::interpolate with FillNaN at m times (method 0 Hermite, 1 Legendre);
// returns the number of times outside the orbit.
int64_t ref_orbit_interpolate(const double* sv_pos, const double* sv_vel, int n, double first, double spacing,
                              int method, const double* t, int64_t m, double* pos, double* vel) {
    const RefOrbit orb(sv_pos, sv_vel, n, first, spacing, method);
    int64_t outside = 0;
    for (int64_t k = 0; k < m; ++k) {
        Vec3 p, v;
        const auto st = orb.interpolate(&p, &v, t[k], OrbitInterpBorderMode::FillNaN);
        if (st != isce3::error::ErrorCode::Success) ++outside;
        for (int d = 0; d < 3; ++d) {
            pos[3 * k + d] = p[d];
            vel[3 * k + d] = v[d];
        }
    }
    return outside;
}

// Ellipsoid::lonLatToXyz at m points (lon, lat in radians, height in m).
void ref_lonlat_to_xyz(double a, double e2, const double* llh, int64_t m, double* xyz) {
    const isce3::core::Ellipsoid ell(a, e2);
    for (int64_t k = 0; k < m; ++k) {
        const Vec3 x = ell.lonLatToXyz(Vec3(llh[3 * k], llh[3 * k + 1], llh[3 * k + 2]));
        for (int d = 0; d < 3; ++d) xyz[3 * k + d] = x[d];
    }
}

// isce3::geometry::geo2rdr as geocodeSlc calls it (geometry/geometry.cpp:241-251:
// t0 = the incoming azimuth time, Geo2RdrParams{threshold, maxIter,
// deltaRange}, converged = status Success) over m points; the image-grid
// Doppler is a table without data whose reference value is dop_ref.
// side: -1 right, 1 left.  status[k] = the detail::geo2rdr ErrorCode.
void ref_geo2rdr(const double* sv_pos, const double* sv_vel, int n, double first, double spacing, int method,
                 double a, double e2, const double* llh, int64_t m, double wvl, int side, double t_guess,
                 double threshold, int maxiter, double delta_range, double dop_ref, int bounds_error, double* t_out,
                 double* r_out, int* status) {
    const RefOrbit orb(sv_pos, sv_vel, n, first, spacing, method);
    const isce3::core::Ellipsoid ell(a, e2);
    const ConstDoppler dop{dop_ref, bounds_error != 0};
    const auto look = side < 0 ? isce3::core::LookSide::Right : isce3::core::LookSide::Left;
    const isce3::geometry::detail::Geo2RdrParams params{threshold, maxiter, delta_range};
    for (int64_t k = 0; k < m; ++k) {
        double t = t_guess, r = 0.0;
        const double t0 = t;
        const auto st = isce3::geometry::detail::geo2rdr(&t, &r, Vec3(llh[3 * k], llh[3 * k + 1], llh[3 * k + 2]),
                                                        ell, orb, dop, wvl, look, t0, params);
        t_out[k] = t;
        r_out[k] = r;
        status[k] = (int)st;
    }
}

// UTM::inverse (core/Projections.cpp:202-232) at m points: easting, northing
// in m -> lon, lat in radians; returns the number of failed inversions.
int64_t ref_utm_inverse(int epsg, const double* xy, int64_t m, double* lonlat) {
    const isce3::core::UTM utm(epsg);
    int64_t bad = 0;
    for (int64_t k = 0; k < m; ++k) {
        Vec3 llh;
        const int st = utm.inverse(Vec3(xy[2 * k], xy[2 * k + 1], 0.0), llh);
        if (st != 0) ++bad;
        lonlat[2 * k] = llh[0];
        lonlat[2 * k + 1] = llh[1];
    }
    return bad;
}

// UTM::forward (core/Projections.cpp:171-200): lon, lat in radians -> m.
int64_t ref_utm_forward(int epsg, const double* lonlat, int64_t m, double* xy) {
    const isce3::core::UTM utm(epsg);
    int64_t bad = 0;
    for (int64_t k = 0; k < m; ++k) {
        Vec3 out;
        const int st = utm.forward(Vec3(lonlat[2 * k], lonlat[2 * k + 1], 0.0), out);
        if (st != 0) ++bad;
        xy[2 * k] = out[0];
        xy[2 * k + 1] = out[1];
    }
    return bad;
}

}  // extern "C"
