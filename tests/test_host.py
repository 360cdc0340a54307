"""Host-side mirror of the pyofss interface: grids, pulses, operator tables, ABI."""

import ctypes as ct
import os
import re
import shutil

import numpy as np
import pytest

import golden_cases as gc
from oracle import gnlse_oracle as go
from pyofsschanged_gb300 import Domain, Gaussian, Sech
from pyofsschanged_gb300 import field as pf
from pyofsschanged_gb300.operators import GridTables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("kw", [dict(bit_width=32.0, samples_per_bit=1024),
                                dict(bit_width=12.5, samples_per_bit=8192, centre_nu=359.0),
                                dict(total_bits=4, bit_width=25.0, samples_per_bit=512)])
def test_domain_matches_oracle(kw):
    d, g = Domain(**kw), go.Grid(**kw)
    for a in ("t", "nu", "omega", "Lambda"):
        np.testing.assert_array_equal(getattr(d, a), getattr(g, a))
    assert d.dt == g.dt and d.window_t == g.window_t and d.centre_omega == g.centre_omega


def test_domain_range_checks():
    from pyofsschanged_gb300.domain import OutOfRangeError
    with pytest.raises(OutOfRangeError):
        Domain(centre_nu=100.0)
    with pytest.raises(OutOfRangeError):
        Domain(samples_per_bit=0)


@pytest.mark.parametrize("name", [n for n in gc.names() if n != "sc_cfg_8192"])
def test_pulses_match_reference_fixture(name):
    case = gc.load(name)
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    p = dict(prm["pulse"])
    cls = Sech if p.pop("kind") == "sech" else Gaussian
    a0 = cls(**p)(d, np.zeros(d.total_samples, complex))
    np.testing.assert_array_equal(a0, case["A0"])


def test_operator_tables_match_oracle():
    case = gc.load("gain_ark4ip_1024")
    prm = case["params"]
    d = Domain(**gc.domain_kwargs(prm))
    fk = gc.fibre_kwargs(prm)
    for k in ("method", "local_error", "traces", "total_steps"):
        fk.pop(k, None)
    g = GridTables(d, beta=fk["beta"], gamma=fk["gamma"], self_steepening=True,
                   use_all="blowwood", small_signal_gain=fk["small_signal_gain"],
                   E_sat=fk["E_sat"], length=fk["length"], lamb0=fk["lamb0"],
                   bandwidth=fk["bandwidth"])
    p = go.Propagator(go.Grid(**gc.domain_kwargs(prm)), **fk)
    np.testing.assert_allclose(g.beta_w, p.factor.imag, rtol=1e-15, atol=0)
    np.testing.assert_allclose(g.hR_re + 1j * g.hR_im, p.nl.h_R, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(g.ss_w, 1.0 + p.nl.omega * p.nl.ss_factor, rtol=1e-15)
    np.testing.assert_allclose(g.gain_profile, p.gain.profile, rtol=1e-15)
    assert g.gain_log == p.gain.gain_log


def test_hollenbeck_table_matches_oracle():
    d = Domain(bit_width=12.5, samples_per_bit=2048, centre_nu=359.0)
    g = GridTables(d, beta=[0, 0, -1.0], gamma=1.0, use_all="hollenbeck")
    nl = go.Nonlinear(go.Grid(bit_width=12.5, samples_per_bit=2048, centre_nu=359.0), 1.0,
                      use_all="hollenbeck")
    np.testing.assert_allclose(g.hR_re + 1j * g.hR_im, nl.h_R, rtol=1e-12, atol=1e-12)


def test_field_helpers_convention():
    rng = np.random.default_rng(0)
    a = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    np.testing.assert_allclose(pf.fft(a), go.fft(a), atol=1e-14)
    np.testing.assert_allclose(pf.ifft(pf.fft(a)), a, atol=1e-13)
    t = np.linspace(-1, 1, 64, endpoint=False)
    assert abs(pf.energy(a, t) - go.energy(a, t)) < 1e-14


def _header_symbols():
    syms = set()
    for h in ("gnlse.h", "sno.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        syms |= set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+((?:gnlse|sno)_\w+)\s*\(", src, re.M))
    return sorted(syms)


def test_abi_library_exports_every_declared_symbol():
    from pyofsschanged_gb300 import _native
    lib_path = _native.LIB_PATH
    if not os.path.exists(lib_path):
        if shutil.which("nvcc") is None:
            pytest.skip("libgnlse.so not built and no nvcc")
        from pyofsschanged_gb300 import build
        build.build()
    lib = ct.CDLL(lib_path)
    syms = _header_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_native.SIGNATURES)
    lib.gnlse_abi_version.restype = ct.c_int
    assert lib.gnlse_abi_version() == 2


@pytest.mark.parametrize("name", ["yb_ark4ip_1024", "yb_fixed_2048"])
def test_yb_tables_match_oracle(name):
    """Amplifier2LevelModel tables (amplifier.py:247-344) in the engine's form against
    the oracle's restatement: gain exponent and inversion weights per frequency."""
    case = gc.load(name)
    prm = case["params"]
    fk = gc.fibre_kwargs(prm)
    d = Domain(**gc.domain_kwargs(prm))
    g = GridTables(d, beta=fk["beta"], gamma=fk["gamma"], use_Yb_model=True, Pp_0=fk["Pp_0"],
                   N=fk["N"], Rr=fk["Rr"], yb_cross_sections=fk["yb_cross_sections"])
    grid = go.Grid(**gc.domain_kwargs(prm))
    o = go.YbGain(grid, fk["Pp_0"], fk["N"], fk["Rr"], *fk["yb_cross_sections"])
    yb = g.yb
    assert not g.gain_on
    np.testing.assert_allclose(yb.alpha_s_N, go.fftshift(o.alpha_s * o.N), rtol=1e-14)
    np.testing.assert_allclose(yb.eta_s, go.fftshift(o.eta_s), rtol=1e-14)
    assert yb.Psat_p == pytest.approx(o.Psat_p, rel=1e-15)
    assert yb.ratio_p == o.ratio_p
    assert yb.alpha_p_N == pytest.approx(o.alpha_p * o.N, rel=1e-15)
    assert yb.eta_p == pytest.approx(o.eta_p, rel=1e-15)
    # the inversion sums of a field equal the oracle's sums over Ps / Psat_s
    rng = np.random.default_rng(3)
    a = case["A0"] * (1.0 + 0.1 * rng.standard_normal(d.total_samples))
    X = d.total_samples * go.fft(a)  # the engine's spectral scale, FFT order
    Ps = go.spectral_power(a) * len(a) * grid.dt / o.Tr
    with np.errstate(divide="ignore", invalid="ignore"):
        x, y = o.ratio_s * Ps / o.Psat_s, Ps / o.Psat_s
    assert np.sum(yb.w_ratio * np.abs(X) ** 2) == pytest.approx(np.sum(x[~np.isnan(x)]), rel=1e-12)
    assert np.sum(yb.w_sat * np.abs(X) ** 2) == pytest.approx(np.sum(y[~np.isnan(y)]), rel=1e-12)


def test_yb_cross_section_table_reading(tmp_path):
    """The reference reads its table with a header line; values interpolate with
    zero outside the table."""
    lam = np.linspace(1000e-9, 1060e-9, 61)
    s12 = 1e-25 * np.exp(-((lam - 1030e-9) / 10e-9) ** 2)
    s21 = 2e-25 * np.exp(-((lam - 1035e-9) / 12e-9) ** 2)
    path = tmp_path / "cs.txt"
    rows = [f"{a:.6E}, {b:.6E}, {c:.6E}" for a, b, c in zip(lam, s12, s21)]
    path.write_text("\n".join(rows) + "\n")
    from pyofsschanged_gb300.operators import Amplifier2LevelModel, read_cross_section_table
    l2, a2, b2 = read_cross_section_table(str(path))
    assert len(l2) == 60 and l2[0] == pytest.approx(lam[1], rel=1e-6)
    d = Domain(bit_width=100.0, samples_per_bit=1024, centre_nu=299792.458 / 1030.0)
    amp = Amplifier2LevelModel(Pp=1.0, N=1.0, Rr=1e-5, cross_sections=str(path)).set_domain(d)
    grid = go.Grid(bit_width=100.0, samples_per_bit=1024, centre_nu=299792.458 / 1030.0)
    o12, o21 = go.yb_cross_sections(grid, str(path))
    np.testing.assert_allclose(amp.sigma12_s, o12, rtol=1e-14, atol=0)
    np.testing.assert_allclose(amp.sigma21_s, o21, rtol=1e-14, atol=0)
    assert np.all(amp.sigma12_s[d.Lambda > 1060.0] == 0.0)


def test_rs_factor_tables_reproduce_the_reference_term():
    """raman_scattering=True (nonlinearity.py:236-248) as the engine's Raman tables: the
    engine's term i gamma' ((1 - f_R)|x|^2 + f_R ifft(hR fft(|x|^2))) x equals the
    oracle's default_f_with_rs term."""
    case = gc.load("rs_ark4ip_1024")
    prm = case["params"]
    fk = gc.fibre_kwargs(prm)
    d = Domain(**gc.domain_kwargs(prm))
    g = GridTables(d, beta=fk["beta"], gamma=fk["gamma"], raman_scattering=True,
                   rs_factor=fk["rs_factor"])
    nl = go.Nonlinear(go.Grid(**gc.domain_kwargs(prm)), fk["gamma"], raman_scattering=True,
                      rs_factor=fk["rs_factor"])
    x = case["A0"]
    p = np.abs(x) ** 2
    hr = g.hR_re + 1j * g.hR_im
    conv = go.ifft(hr * go.fft(p))  # G-(hR/n G+(p)) in pyofss fft terms
    engine_term = 1j * g.gamma * ((1.0 - g.f_R) * p + g.f_R * conv) * x
    np.testing.assert_allclose(engine_term, nl(x), rtol=1e-12, atol=1e-9 * np.abs(nl(x)).max())
    with pytest.raises(NotImplementedError):
        GridTables(d, beta=fk["beta"], gamma=fk["gamma"], raman_scattering=True, self_steepening=True)


def test_fibre_model_options_on_the_cuda_path():
    """Fibre accepts the models the engine runs and refuses the rest at construction."""
    from pyofsschanged_gb300 import Fibre
    Fibre(length=1e-5, beta=[0, 0, -10.0], gamma=100.0, raman_scattering=True, method="cuda_ark4ip")
    Fibre(length=1e-3, beta=[0, 0, 25.0], gamma=5.0, use_Yb_model=True, Pp_0=1.0, N=1.0, Rr=1e-5,
          method="cuda_rk4ip")
    for m in ("ss_simple", "ss_reduced", "ss_symmetric", "ss_sym_rk4", "ss_sym_midpoint", "ss_agrawal",
              "ass_symmetric", "ass_sym_rk4", "ass_agrawal"):
        Fibre(length=1e-5, beta=[0, 0, -10.0], gamma=100.0, method=m)
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-5, gamma=100.0, raman_scattering=True, self_steepening=True)
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, use_Yb_model=True, Pp_0=1.0, N=1.0, Rr=1e-5, method="ss_simple")
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, use_Er_profile=True)
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, method="ss_euler")
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, self_steepening=True, method="ass_symmetric")
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, small_signal_gain=10.0, E_sat=1.0, method="ss_sym_rk4")
    with pytest.raises(NotImplementedError):
        Fibre(length=1e-3, gamma=5.0, self_steepening=True, method="ss_reduced")
    Fibre(length=1e-3, gamma=5.0, self_steepening=True, method="ss_sym_rk4")


def test_engine_method_list_matches_the_plan():
    from pyofsschanged_gb300.engine import METHODS
    assert gc.ENGINE_METHODS == set(METHODS)


def test_large_grid_amplifier_tables_match_oracle():
    """The 2^16-point amplifier configuration (100 ps at 1030 nm, saturable gain with a
    40 nm Lorentzian, Raman and self-steepening): the host tables equal the oracle's."""
    lam = 299792.458 / 1030.0
    d = Domain(bit_width=100.0, samples_per_bit=65536, centre_nu=lam)
    kw = dict(beta=[0.0, 0.0, 25.0, 0.05], gamma=5.0, self_steepening=True, use_all="blowwood",
              small_signal_gain=39.09, E_sat=5.0, lamb0=1030.0, bandwidth=40.0)
    g = GridTables(d, length=3e-3, **kw)
    p = go.Propagator(go.Grid(bit_width=100.0, samples_per_bit=65536, centre_nu=lam), 3e-3, **kw)
    np.testing.assert_allclose(g.beta_w, p.factor.imag, rtol=1e-15, atol=0)
    np.testing.assert_allclose(g.hR_re + 1j * g.hR_im, p.nl.h_R, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(g.ss_w, 1.0 + p.nl.omega * p.nl.ss_factor, rtol=1e-15)
    np.testing.assert_allclose(g.gain_profile, p.gain.profile, rtol=1e-15)
    assert g.gain_log == p.gain.gain_log and g.E_sat == p.gain.E_sat
