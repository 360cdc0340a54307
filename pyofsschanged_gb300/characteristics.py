"""Pulse characteristics of stored traces, as pyofss's Storage records them.

``Storage.update_characts`` (pyofss/modules/storage.py:195-209) appends, per
stored trace, the Simpson energy, the peak temporal power, the temporal peaks,
the FWHM duration of the highest peak, the spectral width, and the dispersion /
nonlinear lengths of ``Fibre.get_dispersion_length`` / ``get_nonlinear_length``
(pyofss/modules/fibre.py:179-187).  Energies and peak powers of all traces are
device reductions over the plan's trace buffer (one pass, all traces at once);
the peak and width rules restate pyofss/field.py:208-298 on the host with
scipy.signal, as the reference computes them.
"""

import numpy as np
import torch
from scipy.signal import find_peaks, peak_widths


def simpson_weights(n, device=None, dtype=torch.float64):
    """scipy's even-N composite Simpson weights (Cartwright last-interval correction)."""
    w = torch.empty(n, dtype=dtype, device=device)
    w[0::2] = 2.0 / 3.0
    w[1::2] = 4.0 / 3.0
    w[0] = 1.0 / 3.0
    if n >= 4:
        w[n - 3] = 4.0 / 3.0 - 1.0 / 12.0
        w[n - 2] = 1.0
        w[n - 1] = 5.0 / 12.0
    return w


def energy_and_peak(traces, dt):
    """traces: [k, n] complex device tensor -> (energies nJ [k], peak powers W [k]) on the host.

    Energy is pyofss.field.energy (field.py:161-172): Simpson over |A|^2 in ps x W, x 1e-3.
    """
    p = traces.abs().double() ** 2
    w = simpson_weights(p.shape[1], device=p.device)
    e = (p @ w) * dt * 1e-3
    return e.cpu().numpy(), p.amax(dim=1).cpu().numpy()


def spectral_power(A):
    """pyofss.field.spectral_power (field.py:60-76): ifftshift(|pyofss fft(A)|^2), fft = numpy ifft."""
    return np.fft.fftshift(np.abs(np.fft.ifft(A)) ** 2)


def get_peaks(P):
    """field.py:281-283"""
    peaks, _ = find_peaks(P, height=0, prominence=(np.amax(P) / 10))
    return peaks


def max_peak_params(P):
    """field.py:208-233: FWHM (samples) of the highest peak, by scipy's peak_widths."""
    peaks, props = find_peaks(P, height=0)
    if len(peaks) == 0:
        return None, None, None, None
    i = int(np.argmax(props["peak_heights"]))
    w, h, l, r = peak_widths(P, [peaks[i]], rel_height=0.5)
    return h[0], w[0], l[0], r[0]


def spectrum_width_params(P, prominence):
    """field.py:236-278: several peaks -> span between the outermost tenth-maximum
    crossings; one peak -> its FWHM; none -> None."""
    def find_x(y, x_peak, left):
        x = np.where(P < y)[0]
        f = x[x < x_peak] if left else x[x > x_peak]
        return int((np.amax(f) if left else np.amin(f)) if len(f) else 0)

    peaks, _ = find_peaks(P, prominence=prominence)
    if len(peaks) > 1:
        h = np.amax(P) / 10
        peaks.sort()
        left, right = find_x(h, peaks[0], True), find_x(h, peaks[-1], False)
        return h, right - left, left, right
    if len(peaks) == 0:
        return None, None, None, None
    w, h, l, r = peak_widths(P, peaks, rel_height=0.5)
    return np.amax(h), w[0], l[0], r[0]


def get_duration(P, dt):
    """field.py:293-298 (the highest peak's FWHM in ps)."""
    _, fwhm, _, _ = max_peak_params(P)
    return None if fwhm is None else fwhm * dt


def get_duration_spec(P, dnu):
    """field.py:286-290 (prominence max/100)."""
    _, fwhm, _, _ = spectrum_width_params(P, np.amax(P) / 100)
    return None if fwhm is None else abs(fwhm) * dnu


def trace_characteristics(traces, domain, gamma, beta_2):
    """The Storage lists for traces [k, n] (device tensor): dict of per-trace lists."""
    e, pmax = energy_and_peak(traces, domain.dt)
    host = traces.cpu().numpy().astype(complex)
    out = {k: [] for k in ("energy_list", "max_power_list", "peaks_list", "duration_list",
                           "spec_width_list", "l_d_list", "l_nl_list")}
    for j, A in enumerate(host):
        P = np.abs(A) ** 2
        dur = get_duration(P, domain.dt)
        out["energy_list"].append(float(e[j]))
        out["max_power_list"].append(float(pmax[j]))
        out["peaks_list"].append(get_peaks(P))
        out["duration_list"].append(dur)
        out["spec_width_list"].append(get_duration_spec(spectral_power(A), domain.dnu))
        out["l_d_list"].append(None if (dur is None or not beta_2) else dur ** 2 / abs(beta_2))
        out["l_nl_list"].append(1.0 / (gamma * pmax[j]) if gamma and pmax[j] > 0 else None)
    return out
