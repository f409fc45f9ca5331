"""CPU-only checks of the C ABI library: it loads, exports every entry point
declared in include/wvgpu.h, and its host-side descriptor (no GPU involved)
reproduces the reference's mode set and dispersion relation bit for bit."""
import ctypes
import os
import re

import numpy as np
import pytest

import wvgpu
from _cases import config_from_case, golden_cases, load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from wvgpu import build
    build.build()
    return wvgpu.load_library()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "wvgpu.h")).read()
    return sorted(set(re.findall(r"\b(wv_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert sorted(wvgpu.exported_symbols()) == declared_symbols()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def _wv_config(cf):
    c = config_from_case(cf)
    return wvgpu.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                               planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                               isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_host_descriptor_matches_reference(lib, name):
    cf = golden_cases()[name]
    g = load_golden(name)
    d = wvgpu.describe_modes(_wv_config(cf))
    assert np.array_equal(d["kMode"], g["desc_kMode"])
    assert np.array_equal(d["lMode"], g["desc_lMode"])
    assert np.array_equal(d["omega"].ravel(), g["desc_omega"])
    assert np.array_equal(d["storageRow"], g["desc_storageRow"])
    assert np.array_equal(d["conjugated"], g["desc_conjugated"])


def test_invalid_configuration_messages(lib):
    cf = golden_cases()["odd_15x13x9"]
    c = _wv_config(cf)
    c.Nj = c.Nz
    with pytest.raises(wvgpu.WVKernelError) as e:
        wvgpu.describe(c)
    assert e.value.code == 1
    assert "Nj must lie in [1,Nz-1]" in str(e.value)
    c = _wv_config(cf)
    c.contractVersion = 3
    with pytest.raises(wvgpu.WVKernelError) as e:
        wvgpu.describe(c)
    assert e.value.code == 1
    c = _wv_config(cf)
    c.latitude = 91.0
    with pytest.raises(wvgpu.WVKernelError):
        wvgpu.describe(c)


def test_large_grid_sizes(lib):
    # 256x256x129: Nj=85, Nkl=11439 (reference descriptor sizes)
    c = wvgpu.Configuration(Nx=256, Ny=256, Nz=129, Nj=85, Lx=800e3, Ly=800e3, Lz=4000.0)
    s = wvgpu.describe(c)
    assert s["Nkl"] == 11439 and s["M"] == 972315
    c = wvgpu.Configuration(Nx=512, Ny=512, Nz=257, Nj=170, Lx=800e3, Ly=800e3, Lz=4000.0)
    assert wvgpu.describe(c)["Nkl"] == 45765
