"""Batched library ARK4IP: the unfused comparator of the fused engine's ensemble solve.

The reference's ARK4IP (pyofss/modules/stepper.py:247-376 over Solver.rk4ip,
solver.py:339-354, with Linearity.default_exp_f, linearity.py:241-256, and
Nonlinearity.default_f_all, nonlinearity.py:201-207) written once for a whole batch of
members on one grid: every pyofss ``fft``/``ifft`` is one cuFFT call (torch.fft) over
all members still propagating, every numpy temporary one batched elementwise kernel, and
each member keeps its own step size h, position z and accept / reject decision as
elements of [B] arrays.  Finished members leave the batch.  This is the best one can do
with library FFTs and no fusion, at the same precision as the engine's plan (complex128
for the fp64 / df plans, complex64 for mixed), so the benchmark's ratio to it measures
what the fused kernels buy over batching alone.

A comparator, not the product: the engine (libgnlse.so) is the path the package runs.
Grids with gain or the Yb model are not handled.
"""

import math

import torch


class BatchedARK4IP:
    """ARK4IP over a batch of fields on one grid (GridTables), one fibre length per field."""

    SAFETY, MAX_FACTOR, MIN_FACTOR, ETA = 0.9, 10.0, 0.2, 5  # stepper.py:133-135, solver.py:71

    def __init__(self, tables, dtype=torch.complex128, device="cuda"):
        g = tables
        if g.gain_on or getattr(g, "yb", None) is not None:
            raise NotImplementedError("the batched comparator has no gain model")
        self.dev = torch.device(device)
        self.cdt = dtype
        self.rdt = torch.float64 if dtype == torch.complex128 else torch.float32
        self.n = g.n
        # beta(w) stays FP64: the phase beta h is formed and reduced in FP64 as the engine does
        self.beta = torch.as_tensor(g.beta_w, dtype=torch.float64, device=self.dev)
        self.alpha = g.alpha
        self.kfac = (1j * g.gamma * torch.as_tensor(
            g.ss_w if g.ss_w is not None else [1.0] * g.n, dtype=torch.float64)).to(self.dev, dtype)
        self.raman = g.hR_re is not None
        if self.raman:
            self.hR = torch.complex(torch.as_tensor(g.hR_re), torch.as_tensor(g.hR_im)).to(self.dev, dtype)
            self.fR = g.f_R
        self.evals = 0

    # pyofss field.fft / field.ifft along the last axis
    @staticmethod
    def fft(a):
        return torch.fft.ifft(a, dim=-1)

    @staticmethod
    def ifft(a):
        return torch.fft.fft(a, dim=-1)

    def linear(self, A, h):
        """exp(h D) in the spectral domain, h per row (default_exp_f, uncached)."""
        ph = torch.remainder(h[:, None] * self.beta[None, :], 2.0 * math.pi)
        mag = torch.exp(-0.5 * self.alpha * h)[:, None].expand_as(ph)
        e = torch.polar(mag, ph).to(self.cdt)
        return self.ifft(e * self.fft(A))

    def nonlinear(self, A):
        """default_f_all (nonlinearity.py:201-207), or SPM with self-steepening factor."""
        p = (A.real * A.real + A.imag * A.imag).to(self.cdt)
        if self.raman:
            conv = self.ifft(self.hR * self.fft(p))
            t = A * (1.0 - self.fR) * p + self.fR * A * conv
        else:
            t = A * p
        return self.ifft(self.kfac * self.fft(t))

    def rk4ip(self, A, h):
        """Solver.rk4ip (solver.py:339-354), h per row."""
        self.evals += A.shape[0]
        hh = 0.5 * h
        hc = h.to(self.rdt)[:, None]
        A_I = self.linear(A, hh)
        k0 = self.linear(hc * self.nonlinear(A), hh)
        k1 = hc * self.nonlinear(A_I + 0.5 * k0)
        k2 = hc * self.nonlinear(A_I + 0.5 * k1)
        k3 = hc * self.nonlinear(self.linear(A_I + k2, hh))
        return (k3 / 6.0) + self.linear(A_I + (k0 + 2.0 * k1 + 2.0 * k2) / 6.0, hh)

    def propagate(self, A, lengths, local_error=1e-6, max_iterations=None, h0=None):
        """Propagate the rows of A ([B, n], time domain) to their lengths (km).

        Returns (fields, attempts per row, iterations run).  ``max_iterations`` bounds
        the batched attempts (a timing sample); unfinished rows keep their state.
        """
        A = A.to(self.dev, self.cdt).clone()
        B = A.shape[0]
        L = torch.as_tensor(lengths, dtype=torch.float64, device=self.dev)
        z = torch.zeros(B, dtype=torch.float64, device=self.dev)
        # stepper.py:256-264 with total_steps = 100, traces = 1
        h = torch.clamp(L / 100.0, max=1e-6) if h0 is None else torch.full_like(L, h0)
        attempts = torch.zeros(B, dtype=torch.int64, device=self.dev)
        active = torch.arange(B, device=self.dev)
        f_eta = 2.0 ** (self.ETA - 1.0)
        fa, fb = f_eta / (f_eta - 1.0), 1.0 / (f_eta - 1.0)
        it = 0
        while active.numel() > 0 and (max_iterations is None or it < max_iterations):
            Aa, za, ha, La = A[active], z[active], h[active], L[active]
            ha = torch.where(za + ha > La, La - za, ha)  # last step truncated (stepper.py:291-292)
            A_half = self.rk4ip(Aa, 0.5 * ha)
            A_fine = self.rk4ip(A_half, 0.5 * ha)
            A_coarse = self.rk4ip(Aa, ha)
            nf = torch.linalg.vector_norm(A_fine, dim=-1).double()
            nd = torch.linalg.vector_norm(A_fine - A_coarse, dim=-1).double()
            bad = ~torch.isfinite(A_fine).all(dim=-1)
            delta = torch.where(nf != 0, nd / torch.where(nf != 0, nf, 1.0), nd)
            delta = torch.where(bad, torch.ones_like(delta), delta)  # relative_local_error
            factor = self.SAFETY * torch.pow(local_error / torch.clamp(delta, min=1e-300), 1.0 / self.ETA)
            h_new = torch.where(delta > 0, ha * torch.clamp(factor, self.MIN_FACTOR, self.MAX_FACTOR),
                                ha * self.MAX_FACTOR)
            acc = delta < 2.0 * local_error
            A_acc = fa * A_fine - fb * A_coarse
            A[active] = torch.where(acc[:, None], A_acc, Aa)
            z[active] = torch.where(acc, za + ha, za)
            h[active] = h_new
            attempts[active] += 1
            done = acc & (za + ha >= La)
            active = active[~done]
            it += 1
        return A, attempts, it
