"""CPU-side checks of the product: the C-ABI library loads and exports every symbol
include/catana_gpu.h declares; host logic (Bessel zeros, argument validation,
containers, KClkk.savetxt) behaves like the reference.  No GPU compute here."""
import ctypes
import os
import re

import numpy as np
import pytest

import catana_gb300 as catana
from catana_gb300 import _lib
from oracle import oracle as O
from conftest import ROOT


def _declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(catana_gpu_\w+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    names = _declared_symbols()
    assert len(names) >= 10
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_flmn_size():
    assert _lib.lib.catana_gpu_flmn_size(32, 32) == 32 * 32 * 33 // 2
    assert _lib.lib.catana_gpu_flmn_size(0, 5) == 0


def test_kln_matches_oracle_bitwise():
    for lmax, nmax, rmax in [(10, 10, 2500.0), (32, 32, 1000.0), (64, 40, 777.0)]:
        assert np.array_equal(catana.compute_kln(lmax, nmax, rmax), O.compute_kln(lmax, nmax, rmax))


def test_spherical_bessel_zeros_api():
    z = catana.besseltools.SphericalBesselZeros(0)
    assert z[0] == pytest.approx(np.pi)
    assert z[1] == pytest.approx(6.283185307179586)
    assert z[2] == pytest.approx(9.42477796076938)
    assert catana.besseltools.SphericalBesselZeros(5)[9] == pytest.approx(38.8836)
    z2 = catana.besseltools.SphericalBesselZeros(2)
    z2.compute_up_to(100)
    with pytest.raises(TypeError):
        catana.besseltools.SphericalBesselZeros()


def test_point_api():
    """point_test.py:5-17."""
    p = catana.Point()
    assert p.cartesian() == (0.0, 0.0, 0.0)
    assert p.spherical() == (0.0, 0.0, 0.0)
    assert np.allclose(p, np.zeros(3))
    p = catana.Point(0, 0, 1)
    assert p.spherical() == (1, 0, 0)
    assert p.cartesian() == pytest.approx((0, 0, 1))


def test_point_container_api():
    """point_test.py:20-43 plus the constructor's error paths (py_basictypes.cpp:83-110)."""
    pc = catana.PointContainer()
    assert np.array(pc).shape == (0, 3)
    pc.add_point(catana.Point())
    assert np.array(pc).shape == (1, 3)
    data = np.arange(9).reshape(3, 3)
    assert np.allclose(catana.PointContainer(data), data)
    pc = catana.PointContainer(np.ones((2, 3)))
    assert np.allclose(pc[0], pc[1]) and np.allclose(pc[0], [1, 1, 1])
    with pytest.raises(IndexError):
        pc[2]
    with pytest.raises(RuntimeError):
        catana.PointContainer(np.ones((2, 3)), "polar")
    with pytest.raises(RuntimeError):
        catana.PointContainer(np.ones(3))
    with pytest.raises(RuntimeError):
        catana.PointContainer(np.ones((2, 4)))
    with pytest.raises(RuntimeError):
        catana.PointContainer(np.asfortranarray(np.ones((4, 3))))
    xyz = np.array([[0, 0, 1], [1, 1, 1], [-380, -800, 200]], dtype=float)
    assert np.allclose(np.array(catana.PointContainer(xyz, "cartesian")), O.cartesian_to_spherical(xyz), rtol=1e-15)


def test_pixelized_container_host_side():
    """point_test.py:46-53 and PixelizedPointContainer.cpp:13-15."""
    with pytest.raises(TypeError):
        catana.PixelizedPointContainer()
    ppc = catana.PixelizedPointContainer(4)
    assert np.all(ppc.get_countmap() == np.zeros(4 ** 2 * 12))
    assert len(ppc) == 12 * 16
    with pytest.raises(ValueError):
        catana.PixelizedPointContainer(255)


def test_sfb_argument_validation():
    pc = catana.PointContainer(np.ones((3, 3)))
    with pytest.raises(TypeError):
        catana.sfb_decomposition(pc, -1, 4, 10.0)
    with pytest.raises(TypeError):
        catana.sfb_decomposition(pc, 4, 70000, 10.0)
    with pytest.raises(TypeError):
        catana.sfb_decomposition(np.ones((3, 3)), 4, 4, 10.0)
    with pytest.raises(ValueError):
        catana.sfb_decomposition(pc, 4, 4, 10.0, precision="half")
    # batched: one value per catalog where lists are given; work items of 128 or 64 complex m
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc, pc], [4, 4, 4], 4, 10.0, verbose=False)
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc], 4, 4, 10.0, verbose=False, mblock=32)


def test_poly_jl_rejected_where_unsupported():
    """CATANA_JL_POLY serves the raw path only: the pixelized and allocation-free
    entry points reject it before touching a device."""
    offs = np.zeros(12 + 1, dtype=np.int64)
    k, c = np.zeros(4), np.zeros(4)
    st = _lib.lib.catana_gpu_sfb_healpix(1, _lib.ptr(offs), None, 2, 2, 10.0, _lib.JL_POLY, _lib.ptr(k),
                                         _lib.ptr(c), None, None)
    assert st == _lib.ERR_ARG and "POLY" in _lib.last_error()
    st = _lib.lib.catana_gpu_sfb_raw_noalloc(None, None, 0, 2, 2, 10.0, _lib.JL_POLY, _lib.ptr(k), _lib.ptr(c),
                                             _lib.ptr(k), None)
    assert st == _lib.ERR_ARG and "POLY" in _lib.last_error()


def test_savetxt_format(tmp_path):
    k = np.array([[1.256637061435917236e-03, 2.5e-3]])
    c = np.array([[1.0, 2.0]])
    r = catana.KClkk(k.copy(), c.copy(), [])
    base = str(tmp_path / "x")
    r.savetxt(base)
    line = open(base + ".k_ln").read().splitlines()[0]
    assert line == "1.256637061435917236e-03 2.500000000000000052e-03"
    assert np.array_equal(np.loadtxt(base + ".c_ln", ndmin=2), c)
    with pytest.raises(ValueError):
        r.k_ln[0, 0] = 1.0


def test_batched_argument_validation():
    """The batched entry point rejects bad records before it touches a device."""
    pc = catana.PointContainer(np.ones((3, 3)))
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc, pc], 4, 4, 10.0, kmax=-1.0, verbose=False)
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc, pc], 4, 4, [10.0, 0.0], verbose=False)
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc, pc], [4], 4, 10.0, verbose=False)
    with pytest.raises(ValueError):
        catana.sfb_decomposition_batched([pc], 4, 4, 10.0, weights=[np.ones(2)], verbose=False)
    assert _lib.lib.catana_gpu_sfb_raw_batched(None, -1, 0, 0.0, None) == _lib.ERR_ARG
    assert _lib.lib.catana_gpu_sfb_raw_batched(None, 0, 0, 0.0, None) == _lib.OK
    assert ctypes.sizeof(_lib.Catalog) == 72


def test_ingest_spec_validation():
    """The ingest entry point rejects bad specs before it touches a device."""
    assert ctypes.sizeof(_lib.IngestSpec) == 88
    sp = _lib.IngestSpec()
    sp.layout = 8  # unknown bit
    n_out = ctypes.c_int64(-1)
    rec = np.zeros((2, 3))
    out = np.zeros((2, 3))
    assert _lib.lib.catana_gpu_ingest(_lib.ptr(rec), 2, ctypes.byref(sp), _lib.ptr(out), ctypes.byref(n_out),
                                      None) == _lib.ERR_ARG
    sp.layout, sp.mask_nside = 0, 3
    sp.mask = rec.ctypes.data
    assert _lib.lib.catana_gpu_ingest(_lib.ptr(rec), 2, ctypes.byref(sp), _lib.ptr(out), ctypes.byref(n_out),
                                      None) == _lib.ERR_ARG
    with pytest.raises(RuntimeError):
        catana.ingest(rec, coordinate_type="polar")


def test_function_interpolator_and_integral_validation():
    """py_basictypes FunctionInterpolator behaviour (besseltools_test.py:39-53) and the
    integrals entry's argument checks (no device needed)."""
    w = lambda r: np.exp(-(r / 40) ** 2) * r ** 2
    fi = catana.FunctionInterpolator(w, 100000, 0, 100)
    assert fi(0) == w(0)
    assert fi(99.9) == pytest.approx(w(99.9))
    for bad in (100, -1, 120):
        with pytest.raises(ValueError):
            fi(bad)
    k = np.ones(2)
    out = np.zeros(2)
    tab = np.ones(2)
    assert _lib.lib.catana_gpu_sbessel_integrals(_lib.ptr(tab), 1, 0.0, 1.0, 0, 1.0, _lib.ptr(k), _lib.ptr(k), 2,
                                                 _lib.ptr(out), None) == _lib.ERR_ARG
    kneg = -np.ones(2)
    assert _lib.lib.catana_gpu_sbessel_integrals(_lib.ptr(tab), 2, 0.0, 1.0, 0, 1.0, _lib.ptr(kneg), _lib.ptr(k), 2,
                                                 _lib.ptr(out), None) == _lib.ERR_ARG


def test_raw_binary_roundtrip(tmp_path):
    """RawBinarySink / RawBinarySource record format: 12- or 24-byte records, no header;
    Cartesian records read back through Point(x, y, z)."""
    pts = O.cartesian_to_spherical(np.random.default_rng(5).normal(size=(500, 3)) * 100)
    f32 = tmp_path / "pts_f32.bin"
    catana.io.write_raw_binary(str(f32), pts, "spherical", np.float32)
    assert f32.stat().st_size == 500 * 12
    back = np.asarray(catana.io.read_raw_binary(str(f32), "spherical", np.float32))
    assert np.array_equal(back, pts.astype(np.float32).astype(np.float64))
    f64 = tmp_path / "pts_c64.bin"
    catana.io.write_raw_binary(str(f64), pts, "cartesian", np.float64)
    assert f64.stat().st_size == 500 * 24
    back = np.asarray(catana.io.read_raw_binary(str(f64), "cartesian", np.float64))
    assert np.allclose(back, pts, rtol=1e-12, atol=1e-12)
