"""GSLC sample codecs on the GPU: the standalone kernels of isce3_gb300.types
and the geocoder's fused complex32 loads / complex32 and truncated-mantissa
stores, bit-exact against the NumPy restatement in oracle/codecs.py
(python/packages/isce3/core/types.py:38-165)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from isce3_gb300 import synth, types  # noqa: E402
from isce3_gb300.batch import BatchTuning, GeocodeBatch, GeocodeRequest  # noqa: E402
from isce3_gb300.core import Poly2d  # noqa: E402
from isce3_gb300.geocode import geocode_slc  # noqa: E402
from oracle import codecs  # noqa: E402

pytestmark = pytest.mark.gpu

if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)


def _specials(n, seed):
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal(n) * 10.0 ** rng.uniform(-9, 6, n)
         + 1j * rng.standard_normal(n) * 10.0 ** rng.uniform(-9, 6, n)).astype(np.complex64)
    sp = np.array([complex(np.nan, 1.0), complex(1.0, np.nan), complex(np.inf, -np.inf), 65520 + 65504j,
                   complex(-0.0, 0.0), 2.0 ** -24 + 1j * 2.0 ** -26, 1 + 2.0 ** -11 + 1j * (1 + 3 * 2.0 ** -11), 0j],
                  np.complex64)
    k = min(n, sp.size)
    z[:k] = sp[:k]
    return z


def _bits16(c32):
    return np.ascontiguousarray(c32).view(np.uint16)


@pytest.mark.parametrize("n", [1, 1000, 3_000_001])
def test_codec_kernels_bit_exact(n):
    z = _specials(n, n)
    ref = codecs.to_complex32(z)
    np.testing.assert_array_equal(_bits16(types.to_complex32(z)), _bits16(ref))
    zt = torch.from_numpy(z).cuda()
    out = types.to_complex32(zt)
    assert out.dtype == torch.complex32
    np.testing.assert_array_equal(out.cpu().view(torch.int16).numpy().view(np.uint16), _bits16(ref))
    back = types.read_c4_dataset_as_c8(ref)
    np.testing.assert_array_equal(back.view(np.uint32), codecs.read_c4_as_c8(ref).view(np.uint32))
    for dtype, bits in ((np.complex64, 10), (np.float32, 5), (np.complex128, 30), (np.float16, 4)):
        with np.errstate(over="ignore"):
            a = (z.astype(dtype) if np.iscomplexobj(np.zeros(1, dtype)) else z.real.astype(dtype)).copy()
        b = a.copy()
        types.truncate_mantissa(a, bits)
        codecs.truncate_mantissa(b, bits)
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
    t = torch.from_numpy(z.copy()).cuda()
    types.truncate_mantissa(t, 10)
    b = z.copy()
    codecs.truncate_mantissa(b, 10)
    np.testing.assert_array_equal(t.cpu().numpy().view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module")
def c1():
    return synth.scene_c1()


def _carriers(carrier):
    if not carrier:
        return {}
    return dict(az_carrier=Poly2d(np.array([[0.3, 1.5e-2, -2e-6]]), 0.0, 0.0, 1.0, 1.0),
                rg_carrier=Poly2d(np.array([[0.0]]), 0.0, 0.0, 1.0, 1.0))


def _geocode(sc, slc, geo_dtype=torch.complex64, carrier=False, **kw):
    g = sc.geogrid
    geo = torch.empty((g.length, g.width), dtype=geo_dtype, device="cuda")
    mask = torch.empty((g.length, g.width), dtype=torch.uint8, device="cuda")
    extra = _carriers(carrier)
    geocode_slc(geo, slc, sc.dem, sc.radar_grid, g, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                sc.ellipsoid, sc.threshold, sc.maxiter, mask_block=mask, **extra, **kw)
    torch.cuda.synchronize()
    return geo, mask


@pytest.mark.parametrize("carrier", [False, True])
def test_complex32_radar_blocks_decode_exactly(c1, carrier):
    """complex32 radar blocks give bit for bit the result of geocoding their
    complex64 decoding (the reference workflow's read_c4_dataset_as_c8 then
    geocode_slc), with and without the carrier deramp."""
    c32 = codecs.to_complex32(c1.slc)
    c64 = codecs.read_c4_as_c8(c32)
    g0, m0 = _geocode(c1, torch.from_numpy(c64).cuda(), carrier=carrier)
    g1, m1 = _geocode(c1, torch.from_numpy(c32.view(np.int32)).cuda().view(torch.complex32), carrier=carrier)
    assert torch.equal(m0, m1)
    assert torch.equal(torch.view_as_real(g0).view(torch.int32), torch.view_as_real(g1).view(torch.int32))
    # host NumPy complex32 input takes the same path
    g2 = np.zeros((c1.geogrid.length, c1.geogrid.width), np.complex64)
    geocode_slc(g2, c32, c1.dem, c1.radar_grid, c1.geogrid, c1.orbit, c1.native_doppler, c1.image_grid_doppler,
                c1.ellipsoid, c1.threshold, c1.maxiter, **_carriers(carrier))
    np.testing.assert_array_equal(g2.view(np.uint32), g0.cpu().numpy().view(np.uint32))


def test_complex32_and_truncated_outputs(c1):
    """complex32 geo blocks hold to_complex32 of the complex64 result, and
    output_nonzero_mantissa_bits gives truncate_mantissa of it, bit for bit
    (NaN fill included)."""
    slc = torch.from_numpy(c1.slc).cuda()
    g0, _ = _geocode(c1, slc)
    ref64 = g0.cpu().numpy()
    g1, _ = _geocode(c1, slc, geo_dtype=torch.complex32)
    np.testing.assert_array_equal(g1.cpu().view(torch.int16).numpy().view(np.uint16),
                                  _bits16(codecs.to_complex32(ref64)))
    g2, _ = _geocode(c1, slc, output_nonzero_mantissa_bits=10)
    t = ref64.copy()
    codecs.truncate_mantissa(t, 10)
    np.testing.assert_array_equal(g2.cpu().numpy().view(np.uint32), t.view(np.uint32))
    h = np.zeros((c1.geogrid.length, c1.geogrid.width), codecs.complex32)
    geocode_slc(h, c1.slc, c1.dem, c1.radar_grid, c1.geogrid, c1.orbit, c1.native_doppler, c1.image_grid_doppler,
                c1.ellipsoid, c1.threshold, c1.maxiter)
    np.testing.assert_array_equal(_bits16(h), _bits16(codecs.to_complex32(ref64)))
    with pytest.raises(ValueError):
        _geocode(c1, slc, output_nonzero_mantissa_bits=24)
    with pytest.raises(ValueError):
        _geocode(c1, slc, geo_dtype=torch.complex32, output_nonzero_mantissa_bits=10)


def test_batch_with_complex32_blocks():
    """The persistent batched kernel decodes and encodes the same way."""
    sc = synth.scene_bursts(seed=5, n_az=2, n_sw=2, grid_px=1200, spacing=30.0, lines=(300, 360),
                            samples=(2400, 2600), device="cuda")
    reqs, outs, ref = [], [], []
    for b in sc.bursts:
        w = b.window
        c32 = codecs.to_complex32(b.slc.cpu().numpy())
        dec = torch.from_numpy(codecs.read_c4_as_c8(c32)).cuda()
        r = torch.empty((w.length, w.width), dtype=torch.complex64, device="cuda")
        geocode_slc(r, dec, sc.dem, b.radar_grid, w, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                    sc.ellipsoid, sc.threshold, sc.maxiter, az_carrier=b.az_carrier, rg_carrier=b.rg_carrier)
        ref.append(codecs.to_complex32(r.cpu().numpy()))
        o = torch.empty((w.length, w.width), dtype=torch.complex32, device="cuda")
        outs.append(o)
        reqs.append(GeocodeRequest(o, torch.from_numpy(c32.view(np.int32)).cuda().view(torch.complex32), sc.dem,
                                   b.radar_grid, w, sc.orbit, sc.native_doppler, sc.image_grid_doppler,
                                   sc.ellipsoid, sc.threshold, sc.maxiter,
                                   dict(az_carrier=b.az_carrier, rg_carrier=b.rg_carrier)))
    batch = GeocodeBatch(reqs, "fp64", BatchTuning(use_graph=True))
    batch.run()
    torch.cuda.synchronize()
    for o, r in zip(outs, ref):
        np.testing.assert_array_equal(o.cpu().view(torch.int16).numpy().view(np.uint16), _bits16(r))
    batch.close()
