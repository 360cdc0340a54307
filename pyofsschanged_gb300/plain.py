"""Plain single-instance GPU RK4IP: the unfused baseline of the fused engine.

This path reproduces the reference's call structure on the GPU, one library
call per reference operation: every pyofss ``fft``/``ifft`` is a cuFFT call
through torch.fft, every numpy temporary a separate elementwise kernel, and
the adaptive stepper reads its error estimate back to the host each attempt
(as ``Stepper.adaptive_stepper`` does in Python, pyofss/modules/stepper.py:295-354).
It is the "plain" denominator of the fused-vs-plain comparison and a
second, independent GPU implementation for cross-checks; the product path is
the fused engine in libgnlse.so.
"""

import math

import torch


class PlainRK4IP:
    def __init__(self, tables, length, dtype=torch.complex128, device="cuda"):
        g = tables
        self.dev = torch.device(device)
        self.cdt = dtype
        rdt = torch.float64 if dtype == torch.complex128 else torch.float32
        self.length = length
        self.npts = g.n
        self.beta = torch.as_tensor(g.beta_w, dtype=torch.float64, device=self.dev)
        self.alpha = g.alpha
        self.factor_gamma = torch.as_tensor(
            g.gamma * (g.ss_w if g.ss_w is not None else 1.0) + 0.0 * g.beta_w, dtype=rdt,
            device=self.dev)
        self.raman = g.hR_re is not None
        if self.raman:
            self.hR = torch.complex(torch.as_tensor(g.hR_re, device=self.dev),
                                    torch.as_tensor(g.hR_im, device=self.dev)).to(dtype)
            self.fR = g.f_R
        if getattr(g, "yb", None) is not None:
            raise NotImplementedError("the plain comparison path has no Yb gain model")
        self.gain = g.gain_on
        if self.gain:
            self.gain_log, self.E_sat, self.glen = g.gain_log, g.E_sat, g.gain_length
            self.profile = torch.as_tensor(g.gain_profile, dtype=rdt, device=self.dev)
            n = g.n
            w = torch.full((n,), 2.0 / 3.0, dtype=torch.float64)
            w[1:n - 2:2] = 4.0 / 3.0
            w[0], w[n - 2], w[n - 3], w[n - 1] = 1.0 / 3.0, 1.0, 4.0 / 3.0 - 1.0 / 12.0, 5.0 / 12.0
            self.simpson = (w * g.dt * 1e-3).to(self.dev, rdt)
        self.evals = 0

    # pyofss field.fft / field.ifft
    def fft(self, a):
        return torch.fft.ifft(a)

    def ifft(self, a):
        return torch.fft.fft(a)

    def linear(self, A, h):
        """Linearity.default_exp_f (linearity.py:241-256)."""
        ph = (self.beta * h).remainder(2.0 * math.pi)
        e = torch.polar(torch.full_like(ph, math.exp(-0.5 * self.alpha * h)), ph).to(self.cdt)
        if self.gain:
            energy = torch.sum(self.simpson * (A.real ** 2 + A.imag ** 2))
            amp = (self.gain_log * h / (2.0 * self.glen)) / (1.0 + energy / self.E_sat) * self.profile
            return self.ifft(torch.exp(amp) * (e * self.fft(A)))
        return self.ifft(e * self.fft(A))

    def n(self, A):
        """Nonlinearity.default_f_all / default_f (nonlinearity.py:201-207,266-267)."""
        p = A.real ** 2 + A.imag ** 2
        if self.raman:
            conv = self.ifft(self.hR * self.fft(p.to(self.cdt)))
            y = A * (1.0 - self.fR) * p + self.fR * A * conv
        else:
            y = A * p
        return self.ifft(1j * self.factor_gamma * self.fft(y))

    def rk4ip(self, A, h):
        """Solver.rk4ip (solver.py:339-354)."""
        self.evals += 1
        hh = 0.5 * h
        A_I = self.linear(A, hh)
        k0 = self.linear(h * self.n(A), hh)
        k1 = h * self.n(A_I + 0.5 * k0)
        k2 = h * self.n(A_I + 0.5 * k1)
        k3 = h * self.n(self.linear(A_I + k2, hh))
        return (k3 / 6.0) + self.linear(A_I + (k0 + 2.0 * (k1 + k2)) / 6.0, hh)

    def fixed(self, A, steps):
        h = self.length / steps
        for _ in range(steps):
            A = self.rk4ip(A, h)
        return A

    def adaptive(self, A, tol=1e-6, h0=None, max_attempts=None):
        """Stepper.adaptive_stepper with step doubling (stepper.py:247-376)."""
        z = 0.0
        h = h0 if h0 else min(self.length / 100.0, 1e-6)
        attempts = 0
        while z < self.length:
            if z + h > self.length:
                h = self.length - z
            while True:
                if max_attempts is not None and attempts >= max_attempts:
                    return A, attempts, False
                attempts += 1
                A_half = self.rk4ip(A, 0.5 * h)
                A_fine = self.rk4ip(A_half, 0.5 * h)
                A_coarse = self.rk4ip(A, h)
                nf = torch.linalg.vector_norm(A_fine)
                delta = float((torch.linalg.vector_norm(A_fine - A_coarse) / nf).item())
                if not math.isfinite(delta):
                    delta = 1.0
                h_temp = h
                h = h_temp * (min(10.0, max(0.2, 0.9 * (tol / delta) ** 0.2)) if delta > 0 else 10.0)
                if delta < 2.0 * tol:
                    z += h_temp
                    A = (16.0 / 15.0) * A_fine - (1.0 / 15.0) * A_coarse
                    break
                if h < 1e-37:
                    raise RuntimeError("Step size is extremely small")
        return A, attempts, True
