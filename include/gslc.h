/*
 * gslc.h — C ABI of the GB300 SLC geocoder (libgslc.so).
 *
 * One fused sm_103a kernel geocodes a complex64 SLC onto a geographic grid:
 * DEM biquintic interpolation, zero-Doppler geo2rdr against a Hermite orbit
 * and a LUT2d Doppler, 8-tap windowed-sinc interpolation with carrier
 * deramp/reramp and native-Doppler demodulation, and geometric flattening.
 *
 * Conventions
 *  - Every entry point returns an int status: 0 success, > 0 an argument
 *    error, < 0 a CUDA or runtime error.  Nothing throws across the ABI and
 *    nothing aborts; gslc_last_error() gives the message.
 *  - Bulk arrays (SLC blocks, outputs, DEM raster, LUT samples, subswath
 *    intervals) are DEVICE pointers.  Orbit state vectors and Poly2d
 *    coefficients are HOST pointers; they are folded into launch parameters.
 *  - Calls are ordered on the stream passed in (a cudaStream_t, may be 0).
 *    One context per host thread; a context may be reused across calls.
 *  - Arrays are C-contiguous row-major.  complex64 is interleaved (re, im).
 */
#ifndef GSLC_H
#define GSLC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSLC_OK 0
#define GSLC_EINVAL 1          /* argument error (ValueError on the Python side) */
#define GSLC_EUNSUPPORTED 2    /* valid in the reference, not provided here */
#define GSLC_EPROJ 3           /* projection inverse failed (reference throws) */
#define GSLC_ECUDA (-1)        /* CUDA runtime error */
#define GSLC_ETIMEOUT (-2)     /* a bounded device-side wait ran out */

typedef struct gslc_ctx gslc_ctx;

/* isce3::core::LUT2d<double> (cxx/isce3/core/LUT2d.h:18-112). */
typedef struct {
    int32_t have_data;      /* 0: default LUT — contains() is true, eval() = ref_value */
    int32_t bounds_error;   /* LUT2d::boundsError() */
    int32_t method;         /* isce3 dataInterpMethod: 0 sinc, 1 bilinear, 2 bicubic, 3 nearest, 4 biquintic */
    int32_t nx, ny;         /* width, length */
    int32_t _pad;
    double x0, y0, dx, dy;  /* x = slant range (m), y = azimuth time (s) */
    double ref_value;
    const double* data;     /* device, ny*nx */
} gslc_lut2d;

/* isce3::core::Poly2d (cxx/isce3/core/Poly2d.h:40-70). */
#define GSLC_POLY_MAX_COEFFS 64
typedef struct {
    int32_t x_order, y_order;   /* -1,-1: default polynomial, evaluates to 0 */
    double x_mean, y_mean, x_norm, y_norm;
    const double* coeffs;       /* host, (y_order+1)*(x_order+1); row i = y power i */
} gslc_poly2d;

/* geocodeSlc's AzRgFunc template argument: LUT2d<double> or Poly2d. */
typedef struct {
    int32_t kind;           /* 0 LUT2d, 1 Poly2d */
    int32_t _pad;
    gslc_lut2d lut;
    gslc_poly2d poly;
} gslc_azrg_func;

/* isce3::product::RadarGridParameters (RadarGridParameters.h). */
typedef struct {
    double sensing_start, wavelength, prf, starting_range, range_pixel_spacing;
    int32_t look_side;      /* -1 right, +1 left */
    int32_t _pad;
    int64_t length, width;
} gslc_radar_grid;

/* isce3::product::GeoGridParameters (GeoGridParameters.h). */
typedef struct {
    double start_x, start_y, spacing_x, spacing_y;
    int32_t width, length, epsg, _pad;
} gslc_geo_grid;

/* isce3::core::Orbit, uniformly sampled (core/Orbit.h, core/Linspace.h). */
typedef struct {
    double t0, spacing;     /* time tag i = t0 + i*spacing (s since reference epoch) */
    int32_t n;
    int32_t method;         /* 0 Hermite (n >= 4), 1 Legendre (n >= 9) */
    const double* pos;      /* host, n*3 (m, ECEF) */
    const double* vel;      /* host, n*3 (m/s) */
} gslc_orbit;

/* A DEM raster as GDAL exposes it to isce3::geometry::DEMRasterToInterpolator
 * (geometry/loadDem.cpp:22-133): the whole raster, its geotransform, EPSG. */
typedef struct {
    int64_t width, length;  /* full raster size */
    double gt[6];           /* GDAL geotransform; rotation terms must be 0 */
    int32_t epsg, _pad;
    /* Device samples of raster pixels [data_y_off, data_y_off + data_length) x
     * [data_x_off, data_x_off + data_width), row stride data_stride floats.
     * The window the geocoder needs must lie inside.  data may be NULL for
     * gslc_compute_dem_window. */
    const float* data;
    int64_t data_x_off, data_y_off, data_width, data_length, data_stride;
} gslc_dem_raster;

/* The DEM window the reference loads for a geogrid (DEMInterpolator::loadDEM,
 * geometry/DEMInterpolator.cpp:29-455), in raster pixel coordinates. */
typedef struct {
    int32_t have_raster;    /* 0: every height is the reference height 0 */
    int32_t wraps;          /* 1: window straddles the DEM file discontinuity */
    int64_t x_off, y_off, width, length;
    double x_start, y_start, dx, dy;   /* pixel-centre start of the window */
} gslc_dem_window;

/* isce3::product::SubSwaths (SubSwaths.h). */
typedef struct {
    int32_t n;              /* number of subswaths; 0 means "every sample is subswath 1" */
    int32_t _pad;
    int64_t length, width;
    const int32_t* valid;   /* device, n*length*2: [start, stop) range samples per line */
} gslc_subswaths;

/* Arguments of isce3::geocode::geocodeSlc, array mode
 * (cxx/isce3/geocode/geocodeSlc.cpp:831-968), with the DEM raster in place of
 * isce3::io::Raster. */
typedef struct {
    gslc_radar_grid radar_grid, sliced_radar_grid;
    gslc_geo_grid geo_grid;
    gslc_orbit orbit;
    gslc_lut2d native_doppler, image_grid_doppler;
    gslc_lut2d az_time_correction, srange_correction;
    gslc_azrg_func az_carrier, rg_carrier;
    double ellipsoid_a, ellipsoid_e2;
    double threshold_geo2rdr;
    int32_t numiter_geo2rdr;
    int32_t flatten, reramp, flatten_with_corrected_srange;
    int64_t first_azimuth_line, first_range_sample;
    float invalid_re, invalid_im;
    int32_t n_blocks;       /* number of (rdr, geo) block pairs sharing the geometry */
    int32_t inplace_deramp; /* 1: deramp rdr blocks in place like the reference; 0: leave them */
    int64_t rdr_length, rdr_width;
    const void* const* rdr_blocks;  /* host array of n_blocks device pointers (complex64) */
    void* const* geo_blocks;        /* host array of n_blocks device pointers (complex64, geo length*width) */
    uint8_t* mask;                  /* device or NULL */
    double* carrier_phase;          /* device or NULL */
    double* flatten_phase;          /* device or NULL */
    double* az_index;               /* device or NULL: radar line coordinate per geo pixel (NaN if invalid) */
    double* rg_index;               /* device or NULL: radar sample coordinate per geo pixel */
    gslc_dem_raster dem;
    int32_t dem_margin;             /* DEM pixels of margin (reference default 50) */
    int32_t geo2rdr_precision;      /* 0 FP64 (reference numerics), 1 float-float where it applies (zero
                                       image-grid Doppler, sensingMid in the orbit span), else FP64; a batch
                                       runs float-float only if every request qualifies */
    const gslc_subswaths* subswaths;  /* host pointer to descriptor, or NULL */
    int32_t rdr_deramped;           /* 1: blocks already carry the deramp of these carriers (resident
                                       stores deramp once); the reramp still applies */
    int32_t _pad2;
    /* Sample formats (the GSLC workflow's codecs, nisar/workflows/gslc.py:185-226,
     * isce3/core/types.py:38-165), applied inside the kernel's loads and stores:
     * rdr_format 0 complex64, 1 complex32 (float16 pairs, decoded exactly);
     * geo_format 0 complex64, 1 complex32 (float32 -> float16 round to nearest
     * even, as numpy's astype), 2 complex64 with all but mantissa_bits mantissa
     * bits zeroed (truncate_mantissa). */
    int32_t rdr_format, geo_format;
    int32_t mantissa_bits, _pad3;
} gslc_geocode_args;

/* A context: the sinc table and error words on `device`.  Creating one also
 * lets the device's default memory pool (which the calls' stream-ordered
 * scratch comes from) keep up to 16 GiB cached between synchronisations
 * (cudaMemPoolAttrReleaseThreshold, process-local; a higher value is kept). */
int gslc_ctx_create(int device, gslc_ctx** out);
int gslc_ctx_destroy(gslc_ctx* ctx);
const char* gslc_last_error(const gslc_ctx* ctx);
const char* gslc_version(void);

/* Host-only: the DEM window the geocoder loads for geo_grid
 * (replaces geometry/loadDem.cpp:22-133 + DEMInterpolator.cpp:29-455). */
int gslc_compute_dem_window(const gslc_dem_raster* dem, const gslc_geo_grid* geo_grid, int32_t margin,
                    gslc_dem_window* out);

/* Host-only: platform position/velocity at time t from the per-interval
 * polynomial form of the Hermite interpolant the kernels evaluate (replaces
 * isce3::core::Orbit::interpolate, core/Orbit.cpp:71-86, for Hermite).
 * Returns GSLC_EINVAL outside the orbit's time span. */
int gslc_orbit_interpolate(const gslc_orbit* orbit, double t, double* pos, double* vel);

/* Host-only: zero-Doppler geo2rdr of one ECEF point (isce3::geometry::geo2rdr,
 * geometry/geometry.cpp:241-251 with geometry/detail/Geo2Rdr.icc:114-179, image
 * grid Doppler zero): the Newton iterations the kernels run, from t_guess.
 * converged = 0 (aztime, slant_range NaN) where the reference returns no
 * convergence, including the look-side check and iterates leaving the orbit. */
int gslc_geo2rdr_zero_doppler(const gslc_orbit* orbit, const double* xyz, double t_guess, int32_t look_side,
                              double threshold, int32_t maxiter, double* aztime, double* slant_range,
                              int32_t* converged);

/* Host-only: the float sinc kernel table (SINC_SUB=8192 phases x 8 taps) the
 * kernels use (core/Sinc2dInterpolator.cpp:12-40, cast to float at use). */
int gslc_sinc_table(float* out);

/* Plain form: geocode one geogrid from n_blocks SLC blocks.
 * Replaces isce3::geocode::geocodeSlc<AzRgFunc>, array mode
 * (cxx/isce3/geocode/geocodeSlc.cpp:831-968; bound to Python as
 * isce3.ext.isce3.geocode._geocode_slc in
 * python/extensions/pybind_isce3/geocode/GeocodeSlc.cpp:218-334). */
int gslc_geocode_slc(gslc_ctx* ctx, const gslc_geocode_args* args, void* stream);

/* gslc_geocode_slc with the results delivered to host memory: args' geo
 * blocks and mask (device) are filled as gslc_geocode_slc fills them, and
 * each geo block (geo_format's bytes per pixel) and the mask (if host_mask
 * and args->mask are set) are also copied to host_geo_blocks[b] and
 * host_mask.  The geogrid runs in row bands whose copies proceed on a
 * context-owned stream while the next bands compute; results are those of
 * gslc_geocode_slc bit for bit (band edges fall on tile edges).  Returns
 * after the copies completed.  Page-locked host buffers let the copies
 * overlap; pageable ones are copied too, without overlap.  Serves the same
 * reference call as gslc_geocode_slc (geocodeSlc.cpp:831-968, whose
 * outputs are host arrays) for callers holding host outputs. */
int gslc_geocode_slc_to_host(gslc_ctx* ctx, const gslc_geocode_args* args, void* const* host_geo_blocks,
                             uint8_t* host_mask, void* stream);

/* Raster mode of geocodeSlc (geocode/geocodeSlc.cpp:605-828 and
 * python/extensions/pybind_isce3/geocode/GeocodeSlc.cpp:26-102, whose
 * rasters are GDAL datasets): rdr_blocks are the input raster's bands over
 * the whole radar grid (rdr_length x rdr_width = the grid, first_azimuth_line
 * and first_range_sample 0), geo_blocks the output raster's bands over the
 * whole geogrid, carrier_phase / flatten_phase optional output rasters.  The
 * geogrid is processed in blocks of lines_per_block lines (the reference's
 * default is 1000), each with the DEM window of that block alone
 * (DEMRasterToInterpolator with the block's lines, :653-656); pixels without
 * a result hold invalid_value and the phase rasters invalid_value's real
 * part.  The DEM samples must cover every block's window.  A mask, when
 * given, is written as in array mode (the reference's raster mode has
 * none).  Synchronises the stream. */
int gslc_geocode_slc_raster(gslc_ctx* ctx, const gslc_geocode_args* args, int32_t lines_per_block, void* stream);

/* gslc_geocode_slc for radar blocks (and optionally a DEM window) in host
 * memory, uploaded while the geogrid computes.  Serves the same reference
 * call (geocodeSlc.cpp:831-968 on host arrays) for callers holding host
 * inputs.  args' radar blocks and DEM samples are device buffers of the
 * same shapes that the call fills: the geogrid runs in `bands` row bands
 * (0: 6); each band's radar lines and DEM rows are planned on the host from
 * the zero-Doppler geometry of its perimeter at -500 m and 9000 m (plus
 * `margin` lines and rows; a negative margin shrinks the plan), uploaded in
 * band order on a context stream with the carrier deramp of each chunk, and
 * the band's kernel starts when they have arrived, on one of two streams
 * that alternate so that band tails overlap.  Everything is uploaded by the
 * end of the call.  A sinc chip or DEM spline that reaches beyond what had
 * arrived is flagged by the kernel and every band runs again once all has
 * arrived (gslc_last_io_reruns reports it), so the results equal
 * gslc_geocode_slc's on the same inputs whatever the plan.  Outputs stay in
 * args' device buffers and, when geo_blocks is given, are also copied to host
 * memory band by band.  Host buffers may be pageable; page-locked ones let
 * the copies overlap fully.  Not with inplace_deramp.  Synchronises the
 * stream. */
typedef struct {
    const void* const* rdr_blocks;  /* n_blocks host radar blocks, args' shape and sample format */
    const float* dem;               /* host samples at the first row and column of the DEM window that args->dem's
                                       device samples hold, or NULL when those are on the device already */
    int64_t dem_stride;             /* row stride of dem, in samples */
    void* const* geo_blocks;        /* n_blocks host outputs (args' geo_format), or NULL */
    uint8_t* mask;                  /* host mask output (needs args->mask), or NULL */
    int32_t bands;                  /* geogrid row bands; 0: 6 */
    int32_t margin;                 /* extra radar lines and DEM rows planned around each band */
} gslc_host_io;

int gslc_geocode_slc_host_io(gslc_ctx* ctx, const gslc_geocode_args* args, const gslc_host_io* io, void* stream);
/* 1 if the last gslc_geocode_slc_host_io call on ctx ran its bands again. */
int gslc_last_io_reruns(const gslc_ctx* ctx);

/* carrierPhaseDeramp (cxx/isce3/geocode/geocodeSlc.cpp:240-274) on its own:
 * dst = src * exp(-i float(rg_carrier(t, r) + az_carrier(t, r))) for a
 * length x width block starting at (first_line, first_sample) of radar_grid.
 * src == dst works in place.  With zero carriers it copies.  Resident stores
 * deramp an SLC once and then geocode it with rdr_deramped = 1. */
int gslc_deramp_block(gslc_ctx* ctx, const gslc_radar_grid* radar_grid, const gslc_azrg_func* az_carrier,
                      const gslc_azrg_func* rg_carrier, int64_t first_line, int64_t first_sample,
                      const void* src, void* dst, int64_t length, int64_t width, void* stream);

/* The GSLC workflow's sample codecs on device arrays of n complex samples
 * (python/packages/isce3/core/types.py:38-72, used by
 * nisar/workflows/gslc.py:185-226): complex64 -> complex32 with numpy's
 * float32 -> float16 rounding (to_complex32), complex32 -> complex64
 * (read_c4_dataset_as_c8, exact), and truncate_mantissa (types.py:116-165)
 * on n_words float16, float32 or float64 words (word_bytes 2, 4, 8) in place. */
int gslc_complex64_to_complex32(gslc_ctx* ctx, const void* src, void* dst, int64_t n, void* stream);
int gslc_complex32_to_complex64(gslc_ctx* ctx, const void* src, void* dst, int64_t n, void* stream);
int gslc_truncate_mantissa(gslc_ctx* ctx, void* data, int64_t n_words, int32_t word_bytes, int32_t significant_bits,
                           void* stream);

/* Host-only: the DEM window of geogrid lines [line_start, line_start +
 * block_length) x [0, block_width) (the block form of
 * DEMRasterToInterpolator, geometry/loadDem.cpp:22-133). */
int gslc_compute_dem_window_block(const gslc_dem_raster* dem, const gslc_geo_grid* geo_grid, int32_t line_start,
                                  int32_t block_length, int32_t block_width, int32_t margin, gslc_dem_window* out);

/* Arguments of isce3::cuda::geocode::Geocode (constructor + geocodeRasters,
 * cxx/isce3/cuda/geocode/Geocode.h:70-128): complex64 rasters on the radar
 * grid of a RadarGeometry, sinc-interpolated onto one geogrid. */
typedef struct {
    gslc_radar_grid radar_grid;     /* RadarGeometry::radarGrid() */
    gslc_geo_grid geo_grid;
    gslc_orbit orbit;               /* RadarGeometry::orbit() */
    gslc_lut2d doppler;             /* RadarGeometry::doppler(): the geo2rdr Doppler */
    gslc_lut2d native_doppler, az_time_correction, srange_correction;
    gslc_dem_raster dem;
    const gslc_subswaths* subswaths;  /* host pointer to descriptor, or NULL */
    double ellipsoid_a, ellipsoid_e2;
    double threshold, delta_range;  /* reference defaults 1e-8, 10 */
    int32_t maxiter;                /* reference default 50 */
    int32_t lines_per_block;        /* reference default 1000 */
    int32_t n_rasters;
    int32_t geo2rdr_precision;      /* 0 FP64, 1 float-float */
    const void* const* input_rasters;   /* host array of device pointers (complex64, radar length*width) */
    void* const* output_rasters;        /* host array of device pointers (complex64, geo length*width) */
    const double* invalid_values;       /* host, n_rasters: output is (v, v) where invalid */
    double* az_index;               /* device or NULL: radar line coordinate per geo pixel (NaN if masked) */
    double* rg_index;               /* device or NULL */
    int32_t dem_margin;             /* DEM pixels of margin per block (reference: 50) */
    int32_t _pad;
} gslc_raster_geocode_args;

/* Geocode rasters block by block with the CUDA geocoder's rules
 * (Geocode::geocodeRasters, cxx/isce3/cuda/geocode/Geocode.cu:652-864, for
 * SINC_METHOD and GDT_CFloat32; bound to Python as
 * isce3.cuda.geocode.Geocode.geocode_rasters,
 * python/extensions/pybind_isce3/cuda/geocode/cuGeocode.cpp:17-90).  Each
 * geogrid block of lines_per_block lines has its own DEM window, as there. */
int gslc_geocode_rasters(gslc_ctx* ctx, const gslc_raster_geocode_args* args, void* stream);

/* One raster interpolated at per-pixel radar coordinates: the interpolate
 * kernel of the CUDA raster geocoder (cxx/isce3/cuda/geocode/Geocode.cu:203-287
 * with the device interpolators of cxx/isce3/cuda/core/: sinc, bilinear,
 * bicubic, nearest, biquintic) for every data type it accepts.  az_index and
 * rg_index (device, n_px doubles) are the radar line and sample of each
 * geogrid pixel as gslc_geocode_rasters writes them (NaN where masked);
 * raster is the device raster (length x width samples), out n_px samples of
 * the same type.  gdal_type: GDALDataType code (1 Byte, 2 UInt16, 4 UInt32,
 * 6 Float32, 7 Float64, 10 CFloat32, 11 CFloat64); method: isce3
 * dataInterpMethod (0 sinc, 1 bilinear, 2 bicubic, 3 nearest, 4 biquintic;
 * integer types nearest only, GSLC_EINVAL otherwise).  Masked pixels and
 * pixels within 4 samples of the raster's edge take invalid_value (both
 * parts for complex types).  Enqueued on stream, not synchronised.  A
 * gslc_geocode_rasters call with n_rasters = 0 and az_index / rg_index set
 * computes the coordinates alone. */
int gslc_interpolate_raster(gslc_ctx* ctx, const double* az_index, const double* rg_index, int64_t n_px,
                            const void* raster, int64_t length, int64_t width, void* out, int32_t gdal_type,
                            int32_t method, double invalid_value, void* stream);

/* Number of the library's own kernels launched by the last call on ctx. */
int64_t gslc_last_launch_count(const gslc_ctx* ctx);

/* Measurement: when enabled, each geocode call records CUDA events on its
 * stream around the fused geocode kernel(s) and the deramp pre-pass;
 * gslc_last_kernel_ms reads their durations after the call returns. */
int gslc_ctx_set_timing(gslc_ctx* ctx, int32_t enable);
int gslc_last_kernel_ms(const gslc_ctx* ctx, float* geocode_ms, float* deramp_ms);

/* Failure handling of the one device-side wait: each block of the fused and
 * persistent kernels copies the orbit's Newton tables into shared memory
 * (cp.async.bulk, an mbarrier counting the bytes) and every thread waits for
 * them at most `clocks` SM clocks (default, and for clocks <= 0: 2^31,
 * about a second).  A thread whose wait runs out reads the tables from
 * global memory instead, so the outputs stay complete and identical, and
 * the call returns GSLC_ETIMEOUT; before a block finishes one thread waits
 * (bounded) for its copy still in flight.  No counterpart in the reference,
 * whose kernels do not stage (cuda/geocode/Geocode.cu:87-287); the setting
 * exists so that the failure path can be exercised. */
int gslc_ctx_set_stage_wait(gslc_ctx* ctx, int64_t clocks);

/* Measurement: sustained FP64 FMA rate of this GPU (GFLOP/s, 2 flops per
 * FMA) from a dependent-chain DFMA loop over all SMs; the denominator of the
 * FP64 roofline the geocode kernel is reported against. */
int gslc_probe_fp64_gflops(gslc_ctx* ctx, double* gflops);

/* Batched form.  A batch holds many geocode requests (bursts, tiles of
 * uneven size; each a gslc_geocode_args with its own radar grid, radar
 * blocks, geogrid window and outputs).  One launch runs the deramp passes and
 * either ONE persistent kernel whose blocks pop runs of 32 x 8/16/32-pixel
 * tiles of any request from a device counter, or (tuning per_request) each
 * request's own fused kernel on up to four branch streams forked from and
 * joined into the launch stream; by default the whole sequence is captured
 * in a CUDA graph at creation (the branches as parallel paths) and replayed
 * by gslc_batch_launch.  Each request's outputs equal its plain
 * gslc_geocode_slc call (with 32 x 32 tiles: rows_per_thread 4).  Pointers in the
 * requests are bound at creation: relaunching recomputes the same outputs
 * from the (possibly updated) contents of the same buffers.  No counterpart
 * in the reference, which geocodes one block per call
 * (geocodeSlc.cpp:831-968, driven block by block by
 * python/packages/nisar/workflows/gslc.py:173-214). */
typedef struct gslc_batch gslc_batch;
typedef struct {
    int32_t tiles_per_pop;   /* tiles a block takes per counter pop; 0: 2 */
    int32_t blocks_per_sm;   /* persistent blocks per SM; 0: occupancy maximum */
    int32_t use_graph;       /* 1: capture and replay a CUDA graph; 0: launch directly */
    int32_t rows_per_thread; /* geogrid lines per thread: 1, 2 or 4 (tiles of 32 x 8/16/32 pixels); 0: 4 */
    int32_t per_request;     /* 1: each request's own fused kernel (the plain call's, 32 x 32 tiles) on
                                concurrent streams, in place of the persistent queue; the three fields
                                above do not apply */
} gslc_batch_tuning;

/* Device buffers are allocated and filled in the order of `stream`
 * (cudaMallocAsync / cudaMemcpyAsync), so creating, launching and destroying
 * batches never synchronises the device: launch a batch on its creation
 * stream (or after it); destroy releases its buffers in that stream's order. */
int gslc_batch_create(gslc_ctx* ctx, const gslc_geocode_args* requests, int32_t n_requests,
                      int32_t geo2rdr_precision, const gslc_batch_tuning* tuning, void* stream, gslc_batch** out);
/* As gslc_batch_create, with per-request completion: done_flags is
 * n_requests words of mapped host memory (gslc_host_flags_create) set to 1
 * when request i's outputs have been written (by the block writing its last
 * tile, or by a one-thread kernel behind its own kernel), while the rest of
 * the batch still runs.  The caller clears them before a launch. */
int gslc_batch_create_signaled(gslc_ctx* ctx, const gslc_geocode_args* requests, int32_t n_requests,
                               int32_t geo2rdr_precision, const gslc_batch_tuning* tuning, void* stream,
                               uint32_t* done_flags, gslc_batch** out);
/* Mapped, device-visible host words for completion flags (cleared). */
int gslc_host_flags_create(int32_t n, uint32_t** host);
int gslc_host_flags_destroy(uint32_t* host);
int gslc_batch_launch(gslc_batch* batch, void* stream);     /* enqueue only */
int gslc_batch_status(gslc_batch* batch, void* stream);     /* synchronise the stream, report errors */
int gslc_batch_info(const gslc_batch* batch, int64_t* n_tiles, int32_t* blocks, int32_t* tiles_per_pop,
                    int64_t* launches);
int gslc_batch_destroy(gslc_batch* batch);

/* Block planning.  One geogrid block of a geogrid (its own start, same
 * spacing and EPSG), as python/packages/isce3/core/rdr_geo_block_generator.py
 * builds it for each block. */
typedef struct {
    double start_x, start_y, spacing_x, spacing_y;
    int32_t width, length;
} gslc_geo_block;

/* isce3::geometry::RadarGridBoundingBox (geometry/boundingbox.h:18-23) plus
 * the outcome: status 0 ok; 1 geo2rdr did not converge at the corners in
 * `detail` (bit 0 top-left/north-west, 1 top-right, 2 bottom-left, 3
 * bottom-right; the reference's RuntimeError "did not converge"); 2 the box
 * does not overlap the radar grid (bit 0 azimuth first and last <= 0, 1
 * both >= max azimuth, 2 range <= 0, 3 range >= max range; RuntimeError
 * "does not overlap"); 3 a projection inverse failed (RuntimeError
 * "Inverse projection transformation failed"). */
typedef struct {
    int32_t first_azimuth_line, last_azimuth_line, first_range_sample, last_range_sample;
    int32_t status, detail;
} gslc_radar_bbox;

/* Arguments of isce3::geometry::getRadarBoundingBox with min/max heights
 * (geometry/boundingbox.h:152-161). */
typedef struct {
    gslc_radar_grid radar_grid;
    gslc_orbit orbit;
    gslc_lut2d doppler;             /* radar image grid Doppler; default LUT2d: zero */
    int32_t epsg;                   /* of every block: 4326 or UTM */
    int32_t n_blocks;
    const gslc_geo_block* blocks;   /* host, n_blocks */
    float min_height, max_height;
    int32_t margin;                 /* >= 0 */
    int32_t geogrid_expansion_threshold;
    double threshold;               /* Geo2RdrParams: 1e-8 */
    int32_t maxiter, _pad;          /* 50 */
    double delta_range;             /* 10 */
} gslc_bbox_args;

/* The radar bounding box of every block in ONE launch (8 geo2rdr sequences per
 * block, one thread each).  Replaces isce3::geometry::getRadarBoundingBox
 * (geometry/boundingbox.cpp:434-641; bound as
 * isce3.geometry.get_radar_bbox in
 * python/extensions/pybind_isce3/geometry/boundingbox.cpp:82-131) called once
 * per block by block_generator (rdr_geo_block_generator.py:55-117).  `out` is
 * host memory for n_blocks results; the call returns when they are there.
 * Argument errors (max_height < min_height, margin < 0) return GSLC_EINVAL
 * like the reference's InvalidArgument / OutOfRange; per-block failures are
 * statuses, never call errors.  geogrid_expansion_threshold is limited to
 * [0, 10000] and maxiter to [0, 1000] (GSLC_EINVAL beyond), which bounds the
 * work of one thread; the reference has no limit. */
int gslc_radar_bbox_blocks(gslc_ctx* ctx, const gslc_bbox_args* args, gslc_radar_bbox* out, void* stream);

/* DEM statistics over a device float raster (length x width, row stride in
 * floats): min, max and mean of the non-NaN samples and their count.
 * Replaces isce3::geometry::DEMInterpolator::computeMinMaxMeanHeight
 * (geometry/DEMInterpolator.cpp:515-560).  The mean's sum is folded in a
 * fixed order, so it is the same on every call; with no valid sample min is
 * FLT_MAX, max -FLT_MAX and mean NaN, as there. */
int gslc_dem_stats(gslc_ctx* ctx, const float* data, int64_t length, int64_t width, int64_t row_stride,
                   float* min_height, float* max_height, double* mean_height, int64_t* n_valid, void* stream);

/* Arguments of isce3::geometry::makeRadarGridCubes
 * (geometry/metadataCubes.cpp:276-489) for the outputs the GSLC workflow
 * writes (nisar/workflows/h5_prep.py:869-978).  Each output is device memory
 * of n_heights x length x width elements (height-major) or NULL. */
typedef struct {
    gslc_radar_grid radar_grid;
    gslc_geo_grid geo_grid;         /* EPSG 4326 or UTM */
    const double* heights;          /* host, n_heights */
    int32_t n_heights;
    int32_t maxiter;                /* numiter_geo2rdr, [0, 1000] */
    gslc_orbit orbit;
    gslc_lut2d native_doppler;      /* device data */
    gslc_lut2d grid_doppler;        /* device data */
    double threshold;               /* threshold_geo2rdr */
    double delta_range;
    double* slant_range;            /* f64, m */
    double* azimuth_time;           /* f64, s since the orbit's epoch */
    float* incidence_angle;         /* f32, degrees */
    float* los_unit_vector_x;       /* f32, east component, target to sensor */
    float* los_unit_vector_y;       /* f32, north component */
    float* along_track_unit_vector_x;
    float* along_track_unit_vector_y;
    float* elevation_angle;         /* f32, degrees */
    double* ground_track_velocity;  /* f64, m/s */
} gslc_cube_args;

/* Radar grid metadata cubes in one launch, one thread per (height, line,
 * column) point: geo2rdr with the grid Doppler (slant range, azimuth time),
 * geo2rdr with the native Doppler and the vectors of writeVectorDerivedCubes
 * (metadataCubes.cpp:74-274).  Replaces isce3::geometry::makeRadarGridCubes
 * (bound as isce3.geometry.make_radar_grid_cubes,
 * python/extensions/pybind_isce3/geometry/metadataCubes.cpp:16-35).  Points
 * that do not converge are NaN.  The reference starts each point's solves
 * from the previous point's results (a chain through each height layer in
 * row-major order); this call follows that chain by passes: each launch
 * solves every point from the starts implied by the previous pass, until no
 * convergence status changes (at least 2, at most 16 passes;
 * gslc_last_cube_passes reports them), so the validity masks are the
 * reference's.  Where neighbouring points share an azimuth time the
 * reference's solve can stop at its start, so its own times depend on the
 * visiting order by up to the geo2rdr threshold; times here agree with it
 * to that threshold.  The call synchronises the stream.  A failed
 * projection inverse returns GSLC_EPROJ. */
int gslc_make_radar_grid_cubes(gslc_ctx* ctx, const gslc_cube_args* args, void* stream);
int gslc_last_cube_passes(const gslc_ctx* ctx);

/* Allocation-free plain form.  No counterpart in the reference: an addition
 * for callers that must not allocate device memory while they run (serving
 * loops that reserve HBM up front under a fixed budget, hosts that forbid
 * allocation after start-up, frameworks that own the memory pool).  Same
 * arguments, kernels and results as gslc_geocode_slc, but no context: its
 * scratch lives in file-scope device arrays of the library (about 33.1 MiB
 * per GPU that loads it, held until exit):
 *  - the deramped copy of the radar blocks (complex64, written by the
 *    deramp straight from the caller's complex64 or complex32 blocks) when
 *    carriers are present and inplace_deramp is 0: at most 4194304 complex
 *    samples over all blocks;
 *  - orbit polynomials for at most 256 state vectors; the sinc table (in
 *    float for the SLC, in double for sinc-method LUT2d tables); an error
 *    word cleared by every call.
 * Larger inputs are rejected with GSLC_EINVAL and a message in errbuf.  It
 * calls no cudaMalloc, cudaFree or other allocating routine.  The first call
 * on a device (the current one) looks up the arrays' device addresses and
 * uploads the sinc tables synchronously.  Like gslc_geocode_slc, every call
 * synchronises `stream` before it returns (it reads the error word back).
 * All calls share the arrays: calls that overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller.  errbuf
 * (may be NULL) receives the error message, errbuf_len bytes at most. */
int gslc_geocode_slc_noalloc(const gslc_geocode_args* args, void* stream, char* errbuf, size_t errbuf_len);

#ifdef __cplusplus
}
#endif
#endif /* GSLC_H */
