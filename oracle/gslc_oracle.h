/*
 * CPU oracle for SLC geocoding — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain C++17/OpenMP restatement of isce3's array-mode SLC
 * geocoder (cxx/isce3/geocode/geocodeSlc.cpp:55-511, 831-968) and of every
 * callee on that path.  It exists to check the CUDA product path; only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it.  The product never calls it and has no CPU fallback.
 *
 * Parity status: the reference cannot be compiled here (it needs Eigen,
 * GDAL, HDF5 and pyre), so the end-to-end restatement is pinned by the
 * reference's own runnable known-answer data for the pieces on the path
 * (tests/data/interpolator/data.txt for bilinear/biquintic/sinc, the
 * circular-orbit Hermite KAT of tests/cxx/isce3/core/orbit/orbit.cpp:495-552)
 * and by the synthetic lon/lat-as-phase KAT of
 * tests/cxx/isce3/geocode/geocodeSlc.cpp:231-297 restated on synthetic
 * geometry.  The full geocode path itself is "parity unpinned" against a
 * running reference.
 *
 * Numerics follow the reference operation by operation.  Build with
 * -ffp-contract=off (no FMA contraction), like the reference's x86-64 build.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t have_data;      /* 0: default-constructed LUT, eval -> ref_value */
    int32_t bounds_error;   /* LUT2d::boundsError() */
    int32_t method;         /* 1 bilinear, 3 nearest (isce3 dataInterpMethod) */
    int32_t nx, ny;         /* width, length */
    double x0, y0, dx, dy;
    double ref_value;
    const double* data;     /* ny*nx row-major, host */
} orc_lut2d;

typedef struct {
    int32_t x_order, y_order;   /* -1,-1 : default Poly2d (evaluates to 0) */
    double x_mean, y_mean, x_norm, y_norm;
    const double* coeffs;       /* (y_order+1)*(x_order+1), row = y power */
} orc_poly2d;

typedef struct {
    int32_t kind;           /* 0 LUT2d, 1 Poly2d */
    orc_lut2d lut;
    orc_poly2d poly;
} orc_azrg;

typedef struct {
    double sensing_start, wavelength, prf, starting_range, range_pixel_spacing;
    int32_t look_side;      /* -1 right, +1 left (isce3 LookSide) */
    int64_t length, width;
} orc_radar_grid;

typedef struct {
    double start_x, start_y, spacing_x, spacing_y;
    int32_t width, length, epsg;
} orc_geo_grid;

typedef struct {
    double t0, spacing;     /* state-vector time tags: t0 + i*spacing */
    int32_t n;
    int32_t method;         /* 0 Hermite, 1 Legendre */
    const double* pos;      /* n*3 */
    const double* vel;      /* n*3 */
} orc_orbit;

/* A DEM raster as GDAL would expose it: full array + geotransform + EPSG. */
typedef struct {
    const float* data;      /* length*width, row-major */
    int64_t width, length;
    double gt[6];
    int32_t epsg;
} orc_dem_raster;

typedef struct {
    int32_t n;              /* number of subswaths; 0 -> every sample is sw 1 */
    int64_t length, width;
    const int32_t* valid;   /* n * length * 2 : [start, stop) per line */
} orc_subswaths;

typedef struct {
    orc_radar_grid radar_grid, sliced_radar_grid;
    orc_geo_grid geo_grid;
    orc_orbit orbit;
    orc_lut2d native_doppler, image_grid_doppler, az_time_correction, srange_correction;
    orc_azrg az_carrier, rg_carrier;
    double ell_a, ell_e2;
    double threshold_geo2rdr;
    int32_t numiter_geo2rdr;
    int64_t first_azimuth_line, first_range_sample;
    int32_t flatten, reramp, flatten_with_corrected_srange;
    float invalid_re, invalid_im;
    int32_t n_blocks;
    int64_t rdr_length, rdr_width;
    float* const* rdr_blocks;   /* complex64 interleaved; deramped IN PLACE like the reference */
    float* const* geo_blocks;   /* complex64 interleaved, geo length*width */
    uint8_t* mask;              /* may be NULL */
    double* carrier_phase;      /* may be NULL */
    double* flatten_phase;      /* may be NULL */
    orc_dem_raster dem;
    const orc_subswaths* subswaths;  /* may be NULL */
    /* optional diagnostics (NULL to skip): radar coordinates per geo pixel */
    double* out_az_index;
    double* out_rg_index;
    double* out_uncorrected_srange;
    int32_t dem_margin;         /* DEMRasterToInterpolator default: 50 */
    int32_t nthreads;           /* 0: OpenMP default */
    double phase_seconds[4];    /* out: index pass, deramp, interpolate, reramp */
    uint8_t* out_niter;         /* optional: geo2rdr iterations per geo pixel (0 = not solved) */
} orc_geocode_args;

/* Returns 0 on success; >0 argument error (message via orc_last_error). */
int orc_geocode_slc(orc_geocode_args* a);

/* Raster mode of geocodeSlc (geocode/geocodeSlc.cpp:605-828): rdr_blocks
 * are the input raster's bands over the whole radar grid (read only),
 * geo_blocks / carrier_phase / flatten_phase the output rasters over the
 * whole geogrid; processed in blocks of lines_per_block geogrid lines, each
 * with its own DEM window and radar bounding box (+-5 samples). */
int orc_geocode_slc_raster(orc_geocode_args* a, int32_t lines_per_block);

/* isce3::cuda::geocode::Geocode::geocodeRasters for SINC_METHOD and
 * GDT_CFloat32 (cxx/isce3/cuda/geocode/Geocode.cu:87-287, 378-864), restated
 * on the CPU block by block, bounding boxes included. */
typedef struct {
    orc_radar_grid radar_grid;
    orc_geo_grid geo_grid;
    orc_orbit orbit;
    orc_lut2d doppler;          /* RadarGeometry::doppler(): the geo2rdr Doppler */
    orc_lut2d native_doppler, az_time_correction, srange_correction;
    double ell_a, ell_e2;
    double threshold, delta_range;
    int32_t maxiter, lines_per_block;
    int32_t n_rasters, dem_margin;
    const float* const* input_rasters;  /* complex64 interleaved, radar length*width */
    float* const* output_rasters;       /* complex64 interleaved, geo length*width */
    const double* invalid_values;       /* n_rasters */
    orc_dem_raster dem;
    const orc_subswaths* subswaths;     /* may be NULL */
    double* out_az_index;               /* optional: y index per geo pixel, NaN where masked */
    double* out_rg_index;               /* optional: x index per geo pixel, NaN where masked */
    int32_t nthreads;
} orc_raster_args;

int orc_geocode_rasters(orc_raster_args* a);
const char* orc_last_error(void);

/* ---- component entry points used by the pinning tests ---- */
int orc_orbit_interpolate(const orc_orbit* o, double t, double* pos, double* vel);
/* interpolators over a double matrix (ny x nx); method: 1 bilinear, 3 nearest,
 * 4 biquintic (order 6), 5 sinc (8 taps, 8192 phases) */
double orc_interp2d_double(int method, const double* z, int ny, int nx, double x, double y);
/* the same biquintic, in float, as the DEM interpolator runs it */
float orc_spline2d_float(const float* z, int ny, int nx, double x, double y);
double orc_lut2d_eval(const orc_lut2d* l, double y, double x);
int orc_lut2d_contains(const orc_lut2d* l, double y, double x);
double orc_poly2d_eval(const orc_poly2d* p, double y, double x);
/* projections: forward = lon/lat(rad)/h -> map x/y/h; returns 0 on success */
int orc_proj_forward(int epsg, const double* llh, double* xyz);
int orc_proj_inverse(int epsg, const double* xyz, double* llh);
void orc_lonlat_to_xyz(double a, double e2, const double* llh, double* xyz);
/* geo2rdr with LUT2d Doppler; returns 1 on convergence (geometry.cpp:241-251) */
int orc_geo2rdr(const double* llh, double a, double e2, const orc_orbit* orbit,
                const orc_lut2d* doppler, double* aztime, double* srange,
                double wavelength, int look_side, double threshold, int maxiter,
                double delta_range);
/* sinc kernel table (8192 x 8, float-cast as used), for inspection */
void orc_sinc_table(float* out);
/* DEM subset the geocoder loads for a geogrid (loadDem.cpp:22-133) */
int orc_dem_subset(const orc_dem_raster* dem, const orc_geo_grid* g, int margin,
                   int64_t* x_off, int64_t* y_off, int64_t* width, int64_t* length,
                   double* x_start, double* y_start);

/* radar bounding box of a geogrid (geometry/boundingbox.cpp:434-641).  out:
 * first/last azimuth line, first/last range sample, status (0 ok, 1 geo2rdr
 * failed at the corners in bits of out[5], 2 no overlap with the reasons in
 * out[5], 3 projection inverse failed), detail.  Returns >0 on an argument
 * error (the reference throws InvalidArgument / OutOfRange). */
int orc_radar_bbox(const orc_geo_grid* g, const orc_radar_grid* rg, const orc_orbit* orbit,
                   const orc_lut2d* doppler, float min_height, float max_height, int margin,
                   double threshold, int maxiter, double delta_range, int expansion_threshold,
                   int32_t* out);
/* radar grid metadata cubes (geometry/metadataCubes.cpp:276-489): arrays of
 * n_heights x length x width, NaN where geo2rdr did not converge; NULL skips
 * an output.  Returns >0 if a projection inverse failed. */
int orc_radar_grid_cubes(const orc_radar_grid* rg, const orc_geo_grid* g, const double* heights, int n_heights,
                         const orc_orbit* orbit, const orc_lut2d* native_doppler, const orc_lut2d* grid_doppler,
                         double threshold, int maxiter, double delta_range, double* slant_range,
                         double* azimuth_time, float* incidence, float* los_x, float* los_y, float* along_x,
                         float* along_y, float* elevation, double* ground_velocity, int nthreads);
/* the CUDA raster geocoder's interpolation at per-pixel radar coordinates
 * (cuda/geocode/Geocode.cu:203-287 and cuda/core/gpu*Interpolator.cu), NaN
 * coordinates masked; gdal_type 1, 2, 4, 6, 7, 10, 11; method 0 sinc,
 * 1 bilinear, 2 bicubic, 3 nearest, 4 biquintic.  Returns >0 on an
 * unsupported type. */
int orc_interpolate_raster(const double* az, const double* rg, int64_t n, const void* raster, int64_t L,
                           int64_t W, void* out, int gdal_type, int method, double invalid);
/* DEM statistics (geometry/DEMInterpolator.cpp:515-560) */
void orc_dem_stats(const float* z, int64_t length, int64_t width, float* mn, float* mx, double* mean,
                   int64_t* n_valid);

#ifdef __cplusplus
}
#endif
