// Launch parameters shared by the host launcher and the kernels.
#pragma once
#include <cuda_runtime.h>
#include "gslc_math.cuh"

namespace gslc {

constexpr int MAX_BLOCKS = 16;   // (rdr, geo) block pairs per launch

struct Dem {
    const float* data;          // points at raster (y_off, x_off); row stride = stride
    int64_t stride;
    int32_t width, length;      // window size (spline clamps and bounds use these)
    int32_t have_raster, epsg_is_lonlat;
    double x_start, y_start, dx, dy;
    Utm utm;                    // DEM projection when it is UTM
    SplineConst sc;
    // window rows whose samples are on the device (all of them unless the
    // window is still being uploaded); a spline reaching outside raises bit 3
    // of *err (the launch must be repeated once every row has arrived)
    int32_t avail_lo, avail_hi;
    int32_t* err;
};

struct GeoParams {
    // geogrid
    double gx0, gy0, gdx, gdy;
    int32_t gw, gl;
    int32_t geo_is_lonlat, _pad0;
    Utm utm;
    Dem dem;
    double ell_a, ell_e2;
    Orbit orbit;
    // geo2rdr
    double t_mid;               // RadarGridParameters::sensingMid(), initial guess
    int32_t t_mid_in_orbit, maxiter;
    double thr;
    V3 pos0, vel0;              // orbit at t_mid (first Newton iterate is shared)
    V3 n0;                      // vel0 x pos0: look side of rvec is sign(rvec . n0)
    double inv_vv0;             // 1 / |vel0|^2
    // radar grid (full) and sliced grid
    double rg_t0, rg_prf, rg_r0, rg_dr, rg_wvl;
    int64_t rg_len, rg_wid;
    int32_t look_side, _pad1;
    double s_t0, s_stop, s_r0, s_end, s_half_az, s_half_rg;
    // LUTs
    Lut nat_dop, img_dop, az_corr, sr_corr;
    AzRg az_car, rg_car;
    double flat_scale;          // 4.0 * (M_PI / wavelength)
    double inv_prf, two_pi_over_prf;
    int32_t flatten, reramp, use_corr, carriers_zero;
    float inv_re, inv_im;
    float two_pi_over_prf_f, _pad_f;
    int32_t az_corr_on, sr_corr_on;   // the correction LUT can change a value (data, or a nonzero reference value)
    uint64_t thr_bits;                // bits of thr if thr > 0, else 0 (|x| < thr as a magnitude-bit compare)
    int64_t k_s_t0, k_s_stop, k_s_r0, k_s_end;   // dkey of the sliced grid's bounds
    double rg_inv_dr;                 // 1 / rg_dr (correctly rounded), for the quotient's Markstein form
    double az_first_d, rg_first_d;    // az_first, rg_first
    // radar blocks
    int32_t nblk, _pad2;
    int64_t inL, inW, az_first, rg_first;
    const float2* rdr[MAX_BLOCKS];
    float2* geo[MAX_BLOCKS];
    uint8_t* mask;
    double* carrier_out;
    double* flatten_out;
    double* az_out;
    double* rg_out;
    const float* sinc;          // [SINC_SUB][SINC_LEN]
    const int32_t* subsw;       // [n][length][2] or NULL
    int32_t subsw_n, have_subsw;
    int64_t subsw_len, subsw_wid;
    int32_t* err;               // device error word: bit 0 projection inverse failed
    // geo2rdr Doppler derivative step (geocodeSlc passes 1e-8; the raster
    // geocoder's default is 10)
    double dop_dr;
    // raster mode (cuda/geocode/Geocode.cu semantics): first geogrid line of
    // this launch and the invalid value of each raster
    int32_t raster, geo_row0;
    float inv_blk[MAX_BLOCKS];
    // 1: UTM tiles may use the fitted projection inverse
    int32_t tile_fit;
    // sample formats: rdr 0 complex64, 1 complex32; geo 0 complex64,
    // 1 complex32, 2 complex64 keeping mant_bits mantissa bits
    int32_t rdr_c32, geo_fmt, mant_bits;
    int32_t _pad3;
    // SM clocks a thread waits for the orbit tables' copy into shared memory
    // before it reads the global tables instead (error bit 1)
    int64_t stage_wait;
    // radar lines of the blocks (block-relative) on the device; a sinc chip
    // reaching outside raises error bit 3, as for the DEM rows
    int64_t avail_az_lo, avail_az_hi;
    // The native Doppler of the sinc chip from the radar indices (azc, rgc)
    // when chip_dop is set (a bilinear table with data, spanning fewer than
    // 2^21 radar lines and samples): the reference's
    // contains(t0 + azc / prf, r0 + rgc * dr) as order-key intervals of azc
    // and rgc, and the table coordinates in FP32 as
    // (index - origin) * cells per index, the origin (the table's first
    // cell in radar indices) split into an integer and a fraction.
    int32_t chip_dop, _pad4;
    int64_t cd_kaz_lo, cd_kaz_hi, cd_krg_lo, cd_krg_hi;
    int32_t cd_iaz, cd_irg;
    float cd_faz, cd_frg, cd_saz, cd_srg;
};

// default of GeoParams::stage_wait: ~2^31 SM clocks, about a second
constexpr int64_t STAGE_WAIT_DEFAULT = 1ll << 31;

struct DerampParams {
    const float2* src;          // complex64, or complex32 when src_c32
    float2* dst;                // complex64
    int32_t src_c32, _pad;
    int64_t inL, inW, az_first, rg_first;
    double rg_t0, rg_prf, rg_r0, rg_dr, inv_prf;
    AzRg az_car, rg_car;
};

// A batch of requests for the persistent kernel: per-request parameters in
// device memory, the prefix sum of their tile counts, and the tile counter.
struct BatchQueue {
    const GeoParams* items;      // n_items
    const long long* tile_start; // n_items + 1, tile_start[0] = 0
    int32_t n_items, tiles_per_pop;
    long long n_tiles;
    int32_t ppt, _pad;               // geogrid lines per thread of every request's tiles
    long long* counter;          // zeroed before each launch
    // per-request completion (optional: done_flags == nullptr disables it)
    const int32_t* item_request;     // n_items: request of each items[] entry
    const long long* request_tiles;  // n_requests: tiles over all its entries
    unsigned long long* request_done;  // n_requests, zeroed before each launch
    unsigned int* done_flags;        // n_requests, host-mapped: set to 1 when a request's last tile is written
};

// Radar bounding boxes of geogrid blocks (gslc_plan.cu): 8 geo2rdr
// sequences per block, geometry/boundingbox.cpp:434-641.
struct PlanParams {
    const double* blocks;        // n_blocks x (start x, start y, spacing x, spacing y, width, length)
    int32_t n_blocks, geo_is_lonlat;
    Utm utm;
    Orbit orbit;
    Lut dop;                     // image-grid Doppler of geo2rdr
    double ell_a, ell_e2;        // the projection's ellipsoid (WGS84)
    double t_mid, t0, prf, r0, dr, wvl;   // radar grid: sensingMid, sensingStart, ...
    int32_t look_side, maxiter;
    double thr, delta_range;
    float hmin, hmax;
    int32_t margin, expansion;
    int64_t length, width;       // radar grid size
    int32_t* out;                // n_blocks x (first az, last az, first rg, last rg, status, detail)
};

// Radar grid metadata cubes (gslc_plan.cu, geometry/metadataCubes.cpp:276-489):
// n_heights x length x width points; NULL outputs are skipped.
struct CubeParams {
    double gx0, gy0, gdx, gdy;
    int32_t width, length, n_heights, geo_is_lonlat;
    Utm utm;
    const double* heights;       // device, n_heights
    Orbit orbit;
    Lut grid_dop, nat_dop;
    double t_mid, mid_range, wvl, thr, delta_range;
    int32_t look_side, maxiter, want_vectors, _pad;
    double* slant_range;
    double* azimuth_time;
    float* incidence;
    float* los_x;
    float* los_y;
    float* along_x;
    float* along_y;
    float* elevation;
    double* ground_velocity;
    // chain state: starts of this pass, final iterates and statuses out
    // (bit 0 grid-Doppler solve converged, bit 1 native-Doppler solve converged)
    const double* start_grid;
    const double* start_native;
    double* t_grid;
    double* t_native;
    uint8_t* status;
    int32_t* err;                // bit 0: a projection inverse failed
};
cudaError_t launch_radar_grid_cubes(const CubeParams& p, cudaStream_t s, int64_t* launches);

// Raster interpolation from per-pixel radar coordinates (gslc_raster.cu,
// cuda/geocode/Geocode.cu:203-287).  dtype: one of RASTER_*; method: the
// isce3 dataInterpMethod code (0 sinc, 1 bilinear, 2 bicubic, 3 nearest,
// 4 biquintic).
enum { RASTER_F32 = 0, RASTER_C64 = 1, RASTER_F64 = 2, RASTER_C128 = 3, RASTER_U8 = 4, RASTER_U16 = 5, RASTER_U32 = 6 };
struct RasterInterpParams {
    const double* az;            // radar line coordinate per geogrid pixel (NaN: masked)
    const double* rg;            // radar sample coordinate per geogrid pixel
    int64_t n;                   // geogrid pixels
    const void* rdr;             // raster, L x W samples
    int64_t L, W;
    void* out;                   // n samples
    int32_t dtype, method;
    double invalid;
    const void* sinc;            // SINC_SUB x SINC_LEN table in the component type
};
cudaError_t launch_raster_interp(const RasterInterpParams& p, cudaStream_t s, int64_t* launches);

// DEM statistics (geometry/DEMInterpolator.cpp:515-560): min, max, sum of
// the non-NaN samples and the NaN count.
struct DemStats { float mn, mx; double sum; long long nan; };
constexpr int DEM_STATS_BLOCKS = 304;   // fixed: the fold order, hence the sum, does not depend on the GPU

// launchers (gslc_plan.cu)
cudaError_t launch_radar_bbox(const PlanParams& p, cudaStream_t s, int64_t* launches);
size_t dem_stats_scratch_bytes();
cudaError_t launch_dem_stats(const float* z, int64_t length, int64_t width, int64_t stride, void* scratch,
                             DemStats* host_out, cudaStream_t s, int64_t* launches);

// The float-float Newton covers zero image-grid Doppler with the first
// iterate at sensingMid and converged G series; anything else runs in FP64.
inline bool ff_eligible(const GeoParams& p) {
    return p.t_mid_in_orbit && !p.img_dop.have_data && p.img_dop.ref_value == 0.0 && !p.orbit.seg_div &&
           !p.orbit.legendre;
}

// launchers (gslc_kernels.cu)
cudaError_t launch_geocode(const GeoParams& p, int precision, cudaStream_t s, int64_t* launches);
cudaError_t launch_deramp(const DerampParams& p, cudaStream_t s, int64_t* launches);
cudaError_t launch_fill_f64(double* p, int64_t n, double v, cudaStream_t s, int64_t* launches);
cudaError_t launch_set_flag(unsigned int* flag, cudaStream_t s, int64_t* launches);
// op 0: complex64 -> complex32, 1: complex32 -> complex64, 2: keep `bits`
// mantissa bits of n words of word_bytes (4 or 8) at dst, in place
cudaError_t launch_codec(int op, const void* src, void* dst, int64_t n, int bits, int word_bytes, cudaStream_t s,
                         int64_t* launches);
cudaError_t probe_fp64(double* out, int blocks, int iters, cudaStream_t s);
cudaError_t launch_geocode_persistent(const BatchQueue& q, bool lonlat, bool ff, int blocks, cudaStream_t s,
                                      int64_t* launches);
int persistent_blocks_per_sm(bool lonlat, bool ff, int ppt);
constexpr int TILE_X = 32, TILE_Y = 8;   // geogrid pixels per tile at one line per thread

}  // namespace gslc
