"""Batched supercontinuum ensembles: seeded inputs, one plan, one launch graph.

``sc_ensemble`` builds the ragged noise ensemble of the benchmark: members on
2^12, 2^13 or 2^14-point grids (uniform choice) with a common sample spacing
dt = 12.5 ps / 8192 (windows 6.25 / 12.5 / 25 ps, so every grid spans the
same 655 THz around 835 nm), fibre lengths U[5, 20] cm, peak powers
U[2, 15] kW, sech pulses with FWHM U[30, 120] fs, plus one photon per spectral
mode with a seeded uniform random phase.  The fibre is the 835 nm photonic
crystal fibre of the single supercontinuum run (beta_2..beta_10, gamma =
0.11 /W/m, Blow-Wood Raman f_R = 0.18, tau_1 = 12.2 fs, tau_2 = 32 fs,
self-steepening), propagated with ARK4IP at local error 1e-6.

There is no reference counterpart for the noise model or the coherence
measure; both follow Dudley, Genty & Coen, Rev. Mod. Phys. 78, 1135 (2006).
"""

import math

import numpy as np

from .domain import Domain, lambda_to_nu
from .field import fft, fftshift, ifft
from .operators import GridTables
from .pulses import Sech

PLANCK_W_PS2 = 6.62607015e-34 * 1.0e24  # J s -> W ps^2

# beta_k in ps^k/km at 835 nm (the /m values x 1e3), k = 0..10
BETA_835 = [0.0, 0.0, -11.830, 8.1038e-2, -9.5205e-5, 2.0737e-7, -5.3943e-10, 1.3486e-12,
            -2.5495e-15, 3.0524e-18, -1.7140e-21]
FIBRE_835 = dict(beta=BETA_835, gamma=110.0, self_steepening=True, use_all="blowwood",
                 f_R=0.18, tau_1=12.2e-3, tau_2=32.0e-3)
DT = 12.5 / 8192.0


def one_photon_noise(domain, rng):
    """One photon per mode, uniform random phase, as a temporal field (sqrt W).

    With the pyofss normalisation the energy is window_t * sum_k |A_k|^2, so a
    bin holding one photon h nu_k has |A_k| = sqrt(h nu_k / window_t).
    """
    nu = fftshift(domain.nu)
    amp = np.sqrt(PLANCK_W_PS2 * nu / domain.window_t)
    phi = rng.uniform(0.0, 2.0 * math.pi, domain.total_samples)
    return ifft(amp * np.exp(1j * phi))


class Member:
    def __init__(self, n, length, peak_power, fwhm, seed):
        self.n, self.length, self.peak_power, self.fwhm, self.seed = n, length, peak_power, fwhm, seed


def sc_ensemble(n_members=256, seed=20261203, sizes=(4096, 8192, 16384), length_cm=(5.0, 20.0),
                power_kw=(2.0, 15.0), fwhm_fs=(30.0, 120.0), noise=True):
    """Seeded member parameters and input fields of the ragged SC ensemble."""
    rng = np.random.default_rng(seed)
    members = []
    for i in range(n_members):
        n = int(rng.choice(sizes))
        length = rng.uniform(*length_cm) * 1e-5  # km
        p0 = rng.uniform(*power_kw) * 1e3
        fwhm = rng.uniform(*fwhm_fs) * 1e-3  # ps
        members.append(Member(n, length, p0, fwhm, int(rng.integers(0, 2 ** 31))))
    domains = {n: Domain(bit_width=DT * n, samples_per_bit=n, centre_nu=lambda_to_nu(835.0))
               for n in sorted(set(m.n for m in members))}
    fields = []
    for m in members:
        d = domains[m.n]
        a = Sech(peak_power=m.peak_power, width=m.fwhm, using_fwhm=True)(
            d, np.zeros(m.n, complex))
        if noise:
            a = a + one_photon_noise(d, np.random.default_rng(m.seed))
        fields.append(a)
    return members, domains, fields


def ensemble_plan_inputs(members, domains, local_error=1e-6, cluster=None):
    """GridTables per distinct grid and Instance per member, for engine.Plan."""
    from .engine import Instance
    sizes = sorted(domains)
    cluster = cluster or {}
    grids = [GridTables(domains[n], cluster=cluster.get(n, 0), **FIBRE_835) for n in sizes]
    index = {n: i for i, n in enumerate(sizes)}
    inst = [Instance(index[m.n], method="ark4ip", length=m.length, local_error=local_error,
                     weight=expected_attempts(m)) for m in members]
    return grids, inst


def expected_attempts(m):
    """Relative ARK4IP work of a member: attempts grow as L sqrt(P0 T0).

    Step doubling keeps the nonlinear phase per step roughly constant, and the
    spectral bandwidth the steps must resolve grows with the soliton order
    N = sqrt(gamma P0 T0^2 / |beta2|); fitting the FP64 oracle's attempt counts
    of the benchmark ensemble gives exponents (1.01, 0.51, 0.46) for (L, P0, T0).
    """
    t0 = m.fwhm / (2.0 * math.log(1.0 + math.sqrt(2.0)))
    return m.length * math.sqrt(m.peak_power * t0)


def coherence_g12(spectra):
    """|g12| over ensemble spectra (rows, common grid): |<A_i* A_j>_{i!=j}| / <|A|^2>.

    sum_{i != j} A_i* A_j = |sum_i A_i|^2 - sum_i |A_i|^2, so the pair average
    costs O(members).
    """
    s = np.sum(spectra, axis=0)
    p = np.sum(np.abs(spectra) ** 2, axis=0)
    n = spectra.shape[0]
    num = np.abs(np.abs(s) ** 2 - p) / (n * (n - 1))
    den = p / n
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(den > 0, num / den, 0.0)


def shard(members, rank, world):
    """Member indices of one rank: a contiguous block of the members sorted by
    estimated cost (N log N x expected attempts), cut so every rank gets about the
    same total cost.  Members are independent, so the ranks propagate their shards
    with no collective; only ensemble statistics are reduced afterwards."""
    cost = [m.n * math.log2(m.n) * expected_attempts(m) for m in members]
    order = sorted(range(len(members)), key=lambda i: -cost[i])
    total = sum(cost)
    out, acc, r = [[] for _ in range(world)], 0.0, 0
    for i in order:
        # advance to the next rank once this one holds its share (keep >= 1 member each)
        while r < world - 1 and acc >= total * (r + 1) / world and out[r]:
            r += 1
        out[r].append(i)
        acc += cost[i]
    return sorted(out[rank])


def coherence_partial(spectra, n_bins=None):
    """Per-rank sums for coherence_g12: (sum_i A_i, sum_i |A_i|^2, count).

    A rank whose shard is empty (more ranks than members) passes ``n_bins``, the
    spectrum length, and contributes zero sums with count 0."""
    spectra = np.asarray(spectra, dtype=complex)
    if spectra.size == 0:
        if n_bins is None:
            raise ValueError("an empty shard needs n_bins (the spectrum length)")
        return np.zeros(n_bins, complex), np.zeros(n_bins), 0
    return spectra.sum(axis=0), (np.abs(spectra) ** 2).sum(axis=0), spectra.shape[0]


def coherence_from_sums(s, p, n):
    """|g12| from the ensemble sums of coherence_partial, all-reduced over ranks."""
    num = np.abs(np.abs(s) ** 2 - p) / (n * (n - 1))
    den = p / n
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(den > 0, num / den, 0.0)


def coherence_g12_distributed(spectra, group=None, n_bins=None):
    """coherence_g12 over the union of every rank's spectra: one all-reduce of the
    sums (torch.distributed, any backend), so the spectra themselves never move.
    Every rank passes ``n_bins`` (the common spectrum length) when some shard may be
    empty."""
    import torch
    import torch.distributed as dist
    s, p, n = coherence_partial(spectra, n_bins)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    buf = torch.tensor(np.concatenate([s.real, s.imag, p, [float(n)]]), dtype=torch.float64, device=dev)
    dist.all_reduce(buf, group=group)
    b = buf.cpu().numpy()
    k = len(p)
    return coherence_from_sums(b[:k] + 1j * b[k:2 * k], b[2 * k:3 * k], b[-1])


def common_spectra(fields, sizes_min=4096):
    """Spectra of members on the coarsest grid's frequency points (FFT order).

    With a common dt every grid's frequency points contain those of the
    coarsest grid (every n/n_min-th point), so members are compared bin by bin.
    Each spectrum is taken with its time origin t = 0 at index 0 (the field
    rotated by n/2 samples): the grids' windows [-W/2, W/2) differ, and with the
    window's start as origin the spectra of the same pulse on two grids would
    differ by a phase exp(i w dW/2), a sign (-1)^k at the odd common bins.
    """
    out = []
    for a in fields:
        n = len(a)
        spec = fft(np.roll(np.asarray(a, complex), -(n // 2)))
        step = n // sizes_min
        out.append(spec[::step] * step)
    return np.array(out)
