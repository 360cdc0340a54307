"""Spectral neural operator (SNO) surrogate of a fixed fibre segment, with RK4IP fallback.

No pyofss counterpart.  The surrogate maps an input pulse to the field after a
fixed segment of the supercontinuum fibre (``ensemble.FIBRE_835``, 2^13 points
over 12.5 ps at 835 nm).  It works in the interaction picture of the linear
operator D = i beta(w) (lossless fibre): a(z) = F^-1[exp(-z D) F[A(z)]], so the
network predicts the purely nonlinear change a(L) - a(0) of the normalised field
a = A / sqrt(P0), and the linear propagation is applied exactly around it.
Spectral L2 errors are the same in both pictures (exp(-zD) is unitary).

Network (a Fourier neural operator, Li et al., ICLR 2021; the CPU restatement
used by the tests is oracle/sno_oracle.py): lifting of the per-sample features
[Re a, Im a, |a|^2, t] to W channels, L layers of truncated-DFT spectral mixing
(K modes, a real 2W x 2W matrix per mode) plus pointwise mixing and GELU, and a
two-layer projection added to the input field.  Every layer runs on the
library's BF16 tensor-core GEMM (include/sno.h) with FP32 accumulation; the
truncated forward and inverse DFTs are GEMMs against BF16 cos/sin tables.

Prediction with fallback: two networks trained from different seeds; their
mean is the prediction and their disagreement, scaled by a factor calibrated on
held-out solver results, the error estimate.  Members whose estimate exceeds
the tolerance are propagated by the RK4IP engine instead.
"""

import ctypes as ct
import math

import numpy as np
import torch

from . import _native as nat
from .domain import Domain, lambda_to_nu
from .ensemble import FIBRE_835, DT
from .operators import GridTables
from .pulses import Sech

N_POINTS = 8192
WINDOW_PS = 12.5
CENTRE_NM = 835.0
SEGMENT_KM = 5e-5  # 5 cm


def _ptr(t, off=0):
    return None if t is None else t.data_ptr() + off * t.element_size()


def _check(code, what):
    if code != 0:
        raise RuntimeError(f"{what} failed (status {code})")


def gemm_timeouts():
    """GEMM CTAs whose bounded wait for the tensor cores ran out (0 in a healthy run)."""
    lib = nat.lib()
    out = ct.c_uint(0)
    _check(lib.sno_gemm_timeouts(ct.byref(out)), "sno_gemm_timeouts")
    return int(out.value)


def gemm(M, N, K, A, B, C, ta=0, tb=0, lda=None, ldb=None, ldc=None, sA=0, sB=0, sC=0, batch=1,
         alpha=1.0, beta=0.0, bias=None, gelu_out=None, bf16_out=None, sO=0, splits=1, a_off=0, b_off=0,
         c_off=0, o_off=0, stream=None):
    """C = alpha op(A) op(B) + beta C (+ bias) on the BF16 tensor-core kernel (see include/sno.h)."""
    lib = nat.lib()
    s = stream or torch.cuda.current_stream()
    lda = lda if lda is not None else (M if ta else K)
    ldb = ldb if ldb is not None else (K if tb else N)
    ldc = ldc if ldc is not None else N
    go = None if gelu_out is None else _ptr(gelu_out, o_off)
    bo = None if bf16_out is None else _ptr(bf16_out, o_off)
    _check(lib.sno_gemm(M, N, K, ta, tb, _ptr(A, a_off), lda, sA, _ptr(B, b_off), ldb, sB, _ptr(C, c_off),
                        ldc, sC, batch, ct.c_float(alpha), ct.c_float(beta), _ptr(bias), go, bo, sO, splits,
                        s.cuda_stream), "sno_gemm")


def dft_tables(n, modes):
    """BF16 truncated DFT F [2K, n] (rows cos, -sin) and its real inverse G [n, 2K]."""
    k = np.arange(modes)[:, None]
    t = np.arange(n)[None, :]
    ang = 2.0 * np.pi * ((k * t) % n) / n
    F = np.empty((2 * modes, n))
    F[0::2] = np.cos(ang)
    F[1::2] = -np.sin(ang)
    c = np.where(np.arange(modes) == 0, 1.0, 2.0)[:, None] / n
    G = np.empty((n, 2 * modes))
    G[:, 0::2] = (c * np.cos(ang)).T
    G[:, 1::2] = (-c * np.sin(ang)).T
    return F, G


class SpectralNeuralOperator:
    """The network, its FP32 master weights, BF16 copies, gradients and Adam state."""

    CIN = 4

    def __init__(self, n=N_POINTS, width=64, modes=64, layers=4, hidden=128, seed=0, device=None,
                 params=None):
        self.dev = torch.device(device) if device is not None else torch.device("cuda")
        self.n, self.W, self.K, self.L, self.H = n, width, modes, layers, hidden
        if params is None:
            rng = np.random.default_rng(seed)
            cin, W = self.CIN, width
            params = {"P": rng.standard_normal((cin, W)) / math.sqrt(cin), "bp": np.zeros(W)}
            for l in range(layers):
                params["R%d" % l] = rng.standard_normal((modes, 2 * W, 2 * W)) / (2 * W)
                params["Wp%d" % l] = rng.standard_normal((W, W)) / math.sqrt(W)
                params["b%d" % l] = np.zeros(W)
            params["Q1"] = rng.standard_normal((W, hidden)) / math.sqrt(W)
            params["bq1"] = np.zeros(hidden)
            params["Q2"] = np.zeros((hidden, 2))  # starts as the identity map (out = input)
            params["bq2"] = np.zeros(2)
        self.p = {k: torch.tensor(np.asarray(v), dtype=torch.float32, device=self.dev).contiguous()
                  for k, v in params.items()}
        self.p16 = {k: v.to(torch.bfloat16) for k, v in self.p.items()}
        self.g = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.t = 0
        F, G = dft_tables(n, modes)
        self.F16 = torch.tensor(F, dtype=torch.float32, device=self.dev).to(torch.bfloat16).contiguous()
        self.G16 = torch.tensor(G, dtype=torch.float32, device=self.dev).to(torch.bfloat16).contiguous()
        self._bufs = {}

    def state_dict(self):
        return {k: v.detach().cpu().numpy() for k, v in self.p.items()}

    # -- buffers per batch size ---------------------------------------------------
    def _buf(self, B):
        if B in self._bufs:
            return self._bufs[B]
        n, W, K, L, H = self.n, self.W, self.K, self.L, self.H
        R = B * n
        f32 = dict(dtype=torch.float32, device=self.dev)
        b16 = dict(dtype=torch.bfloat16, device=self.dev)
        b = {
            "X16": [torch.empty(R, W, **b16) for _ in range(L + 1)],
            "Z": [torch.empty(R, W, **f32) for _ in range(L)],
            "Xh": torch.empty(B, 2 * K, W, **f32),
            "Xh16": [torch.empty(B, 2 * K, W, **b16) for _ in range(L)],
            "Yh": torch.empty(B, 2 * K, W, **f32),
            "Yh16": torch.empty(B, 2 * K, W, **b16),
            "Zq": torch.empty(R, H, **f32),
            "H16": torch.empty(R, H, **b16),
            "out": torch.empty(R, 2, **f32),
            # backward
            "d16": torch.empty(R, 2, **b16),
            "dH": torch.empty(R, H, **f32),
            "dH16": torch.empty(R, H, **b16),
            "dXa": torch.empty(R, W, **f32),
            "dXb": torch.empty(R, W, **f32),
            "dZ16": torch.empty(R, W, **b16),
            "dYh": torch.empty(B, 2 * K, W, **f32),
            "dYh16": torch.empty(B, 2 * K, W, **b16),
            "dXh": torch.empty(B, 2 * K, W, **f32),
            "dXh16": torch.empty(B, 2 * K, W, **b16),
        }
        self._bufs = {B: b}  # keep one batch size resident
        return b

    # -- forward / backward -----------------------------------------------------
    def forward(self, feat16, resid):
        """feat16: [B*n, 4] bf16; resid: [B*n, 2] float32 -> out [B*n, 2] float32."""
        n, W, K, L, H = self.n, self.W, self.K, self.L, self.H
        R = feat16.shape[0]
        B = R // n
        b = self._buf(B)
        p16 = self.p16
        self._feat16 = feat16
        # lifting: X0 = feat P + bp
        gemm(R, W, self.CIN, feat16, p16["P"], b["Z"][0], bias=self.p["bp"], bf16_out=b["X16"][0])
        for l in range(L):
            X16 = b["X16"][l]
            # truncated DFT per sample: Xh = F X
            gemm(2 * K, W, n, self.F16, X16, b["Xh"], ldb=W, sA=0, sB=n * W, sC=2 * K * W, batch=B,
                 bf16_out=b["Xh16"][l], sO=2 * K * W)
            # per-mode mixing: Yh[b, k, :] = Xh[b, k, :] R[k]   (batched over the K modes)
            gemm(B, 2 * W, 2 * W, b["Xh16"][l], p16["R%d" % l], b["Yh"], lda=2 * K * W, ldb=2 * W,
                 ldc=2 * K * W, sA=2 * W, sB=4 * W * W, sC=2 * W, batch=K, bf16_out=b["Yh16"], sO=2 * W)
            # pointwise mixing + bias, then the inverse truncated DFT added, GELU
            gemm(R, W, W, X16, p16["Wp%d" % l], b["Z"][l], bias=self.p["b%d" % l])
            gemm(n, W, 2 * K, self.G16, b["Yh16"], b["Z"][l], lda=2 * K, ldb=W, ldc=W, sA=0,
                 sB=2 * K * W, sC=n * W, batch=B, beta=1.0, gelu_out=b["X16"][l + 1], sO=n * W)
        gemm(R, H, W, b["X16"][L], p16["Q1"], b["Zq"], bias=self.p["bq1"], gelu_out=b["H16"])
        out = b["out"]
        out.copy_(resid)
        gemm(R, 2, H, b["H16"], p16["Q2"], out, beta=1.0, bias=self.p["bq2"])
        return out

    def backward(self, dout):
        """Accumulate parameter gradients (self.g, zeroed here) for d loss / d out = dout."""
        lib = nat.lib()
        s = torch.cuda.current_stream().cuda_stream
        n, W, K, L, H = self.n, self.W, self.K, self.L, self.H
        R = dout.shape[0]
        B = R // n
        b = self._buf(B)
        p16, g = self.p16, self.g
        for t in g.values():
            t.zero_()
        splits = max(1, min(256, R // 2048))
        _check(lib.sno_to_bf16(_ptr(dout), _ptr(b["d16"]), dout.numel(), s), "sno_to_bf16")
        gemm(H, 2, R, b["H16"], b["d16"], g["Q2"], ta=1, lda=H, beta=1.0, splits=splits)
        _check(lib.sno_colsum(_ptr(dout), R, 2, _ptr(g["bq2"]), s), "sno_colsum")
        gemm(R, H, 2, b["d16"], p16["Q2"], b["dH"], tb=1, ldb=2)
        _check(lib.sno_gelu_backward(_ptr(b["dH"]), _ptr(b["Zq"]), _ptr(b["dH"]), _ptr(b["dH16"]),
                                     b["dH"].numel(), s), "sno_gelu_backward")
        gemm(W, H, R, b["X16"][L], b["dH16"], g["Q1"], ta=1, lda=W, beta=1.0, splits=splits)
        _check(lib.sno_colsum(_ptr(b["dH"]), R, H, _ptr(g["bq1"]), s), "sno_colsum")
        dX, dN = b["dXa"], b["dXb"]
        gemm(R, W, H, b["dH16"], p16["Q1"], dX, tb=1, ldb=H)
        for l in reversed(range(L)):
            # dZ = dX * GELU'(Z)  (in place), BF16 copy for the GEMMs
            _check(lib.sno_gelu_backward(_ptr(dX), _ptr(b["Z"][l]), _ptr(dX), _ptr(b["dZ16"]), dX.numel(), s),
                   "sno_gelu_backward")
            gemm(W, W, R, b["X16"][l], b["dZ16"], g["Wp%d" % l], ta=1, lda=W, beta=1.0, splits=splits)
            _check(lib.sno_colsum(_ptr(dX), R, W, _ptr(g["b%d" % l]), s), "sno_colsum")
            # through the inverse DFT: dYh = G^T dZ per sample
            gemm(2 * K, W, n, self.G16, b["dZ16"], b["dYh"], ta=1, lda=2 * K, ldb=W, sA=0, sB=n * W,
                 sC=2 * K * W, batch=B, bf16_out=b["dYh16"], sO=2 * K * W)
            # per-mode weights and inputs
            gemm(2 * W, 2 * W, B, b["Xh16"][l], b["dYh16"], g["R%d" % l], ta=1, lda=2 * K * W, ldb=2 * K * W,
                 ldc=2 * W, sA=2 * W, sB=2 * W, sC=4 * W * W, batch=K)
            gemm(B, 2 * W, 2 * W, b["dYh16"], p16["R%d" % l], b["dXh"], tb=1, lda=2 * K * W, ldb=2 * W,
                 ldc=2 * K * W, sA=2 * W, sB=4 * W * W, sC=2 * W, batch=K, bf16_out=b["dXh16"], sO=2 * W)
            # dX_l = dZ Wp^T + F^T dXh
            gemm(R, W, W, b["dZ16"], p16["Wp%d" % l], dN, tb=1, ldb=W)
            gemm(n, W, 2 * K, self.F16, b["dXh16"], dN, ta=1, lda=n, ldb=W, ldc=W, sA=0, sB=2 * K * W,
                 sC=n * W, batch=B, beta=1.0)
            dX, dN = dN, dX
        _check(lib.sno_to_bf16(_ptr(dX), _ptr(b["dZ16"]), dX.numel(), s), "sno_to_bf16")
        gemm(self.CIN, W, R, self._feat16, b["dZ16"], g["P"], ta=1, lda=self.CIN, beta=1.0, splits=splits)
        _check(lib.sno_colsum(_ptr(dX), R, W, _ptr(g["bp"]), s), "sno_colsum")
        return g

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        lib = nat.lib()
        s = torch.cuda.current_stream().cuda_stream
        self.t += 1
        for k in self.p:
            _check(lib.sno_adam(_ptr(self.p[k]), _ptr(self.g[k]), _ptr(self.m[k]), _ptr(self.v[k]),
                                _ptr(self.p16[k]), self.p[k].numel(), ct.c_float(lr), ct.c_float(beta1),
                                ct.c_float(beta2), ct.c_float(eps), self.t, ct.c_float(weight_decay), s),
                   "sno_adam")

    def loss(self, out, target, grad=None):
        """Per-sample relative L2 errors (and d mean / d out into grad)."""
        lib = nat.lib()
        B = out.shape[0] // self.n
        err = torch.empty(B, dtype=torch.float32, device=self.dev)
        _check(lib.sno_rel_l2(_ptr(out), _ptr(target), 2 * self.n, B, _ptr(err), _ptr(grad),
                              torch.cuda.current_stream().cuda_stream), "sno_rel_l2")
        return err


# ----------------------------------------------------------------------------
# Data: seeded pulses, the engine's propagations, the interaction picture
# ----------------------------------------------------------------------------
def segment_domain():
    return Domain(bit_width=WINDOW_PS, samples_per_bit=N_POINTS, centre_nu=lambda_to_nu(CENTRE_NM))


def sample_pulses(count, seed, fwhm_fs=(30.0, 200.0), power_kw=(1.0, 20.0), phi2_fs2=(-500.0, 500.0)):
    """Seeded sech pulses with a quadratic spectral phase: (params [count, 3], fields [count, n])."""
    rng = np.random.default_rng(seed)
    dom = segment_domain()
    fw = rng.uniform(*fwhm_fs, count) * 1e-3
    p0 = rng.uniform(*power_kw, count) * 1e3
    phi2 = rng.uniform(*phi2_fs2, count) * 1e-6  # ps^2
    w = 2.0 * np.pi * np.fft.fftfreq(dom.total_samples, dom.dt)  # FFT order, rad/ps
    fields = np.empty((count, dom.total_samples), complex)
    for i in range(count):
        a = Sech(peak_power=p0[i], width=fw[i], using_fwhm=True)(dom, np.zeros(dom.total_samples, complex))
        # pyofss spectrum convention (fft = scipy ifft): phase exp(i phi2 w^2 / 2)
        fields[i] = np.fft.fft(np.exp(0.5j * phi2[i] * w * w) * np.fft.ifft(a))
    return np.stack([fw, p0, phi2], 1), fields


def propagate(fields, length=SEGMENT_KM, precision="mixed", device=None):
    """The engine's ARK4IP (1e-6) propagation of each field through the segment."""
    from .engine import Instance, Plan
    dom = segment_domain()
    grid = GridTables(dom, **FIBRE_835)
    inst = [Instance(0, method="ark4ip", length=length, local_error=1e-6) for _ in range(len(fields))]
    plan = Plan([grid], inst, precision=precision, device=device)
    f = plan.pack(list(fields))
    plan.propagate(f)
    out = plan.unpack(f)
    st = plan.stats()
    return np.stack([x.cpu().numpy().astype(complex) for x in out]), st


class Picture:
    """Interaction picture of the segment's linear operator on the device."""

    def __init__(self, device=None):
        dom = segment_domain()
        g = GridTables(dom, **FIBRE_835)
        self.dev = torch.device(device) if device is not None else torch.device("cuda")
        self.beta = torch.tensor(g.beta_w, dtype=torch.float64, device=self.dev)
        self.t = torch.tensor(np.asarray(dom.t), dtype=torch.float64, device=self.dev)

    def to_ip(self, A, z):
        """a = F^-1[exp(-i z beta) F[A]] in pyofss's convention (fft = numpy ifft)."""
        return torch.fft.fft(torch.exp(-1j * z * self.beta) * torch.fft.ifft(A, dim=-1), dim=-1)

    def from_ip(self, a, z):
        return torch.fft.fft(torch.exp(1j * z * self.beta) * torch.fft.ifft(a, dim=-1), dim=-1)

    def features(self, a):
        """a: [B, n] complex (normalised) -> feat16 [B*n, 4] bf16, resid [B*n, 2] float32."""
        B, n = a.shape
        tn = (self.t / (0.5 * WINDOW_PS)).to(torch.float32)
        feat = torch.stack([a.real.float(), a.imag.float(), (a.abs() ** 2).float(), tn.expand(B, n)], -1)
        resid = torch.stack([a.real.float(), a.imag.float()], -1)
        return feat.reshape(B * n, 4).to(torch.bfloat16).contiguous(), resid.reshape(B * n, 2).contiguous()

    @staticmethod
    def pack(a):
        return torch.stack([a.real.float(), a.imag.float()], -1).reshape(-1, 2).contiguous()

    @staticmethod
    def unpack(x, B):
        x = x.reshape(B, -1, 2).double()
        return torch.complex(x[..., 0], x[..., 1])


def make_dataset(A0, AL, z=SEGMENT_KM, device=None):
    """Normalised interaction-picture inputs a0 and targets aL (complex128 on the device)."""
    pic = Picture(device)
    A0 = torch.as_tensor(A0, dtype=torch.complex128, device=pic.dev)
    AL = torch.as_tensor(AL, dtype=torch.complex128, device=pic.dev)
    scale = A0.abs().amax(dim=1, keepdim=True)
    return pic, A0 / scale, pic.to_ip(AL, z) / scale, scale


def train(net, pic, a0, aL, epochs=20, batch=16, lr=2e-3, seed=0, log=None):
    """Adam on the mean relative L2 error; returns the per-epoch mean training loss."""
    gen = torch.Generator(device="cpu").manual_seed(seed)
    n_s = a0.shape[0]
    hist = []
    steps = max(1, n_s // batch)
    total = epochs * steps
    it = 0
    for ep in range(epochs):
        perm = torch.randperm(n_s, generator=gen)
        acc = 0.0
        for s in range(steps):
            idx = perm[s * batch:(s + 1) * batch].to(a0.device)
            feat16, resid = pic.features(a0[idx])
            target = pic.pack(aL[idx])
            out = net.forward(feat16, resid)
            grad = torch.empty_like(out)
            err = net.loss(out, target, grad)
            net.backward(grad)
            lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * it / total))  # cosine schedule
            net.adam_step(lr_t)
            acc += float(err.mean())
            it += 1
        hist.append(acc / steps)
        if log:
            log(f"epoch {ep} loss {hist[-1]:.4e}")
    return hist


def predict(net, pic, a0, batch=16):
    """Network output (interaction picture, normalised) for every row of a0."""
    outs = []
    for s in range(0, a0.shape[0], batch):
        x = a0[s:s + batch]
        feat16, resid = pic.features(x)
        out = net.forward(feat16, resid)
        outs.append(pic.unpack(out.clone(), x.shape[0]))
    return torch.cat(outs)


def rel_err(a, b):
    return (torch.linalg.vector_norm(a - b, dim=1) / torch.linalg.vector_norm(b, dim=1)).cpu().numpy()


class SurrogateWithFallback:
    """Two networks; prediction = their mean, error estimate = kappa x disagreement.

    ``calibrate`` sets kappa so that the estimate bounds the true error of the
    held-out calibration set at the given quantile; ``__call__`` returns the
    output fields, using the RK4IP engine for every member whose estimate
    exceeds ``tol``.
    """

    def __init__(self, nets, pic, tol=1e-3, kappa=1.0):
        self.nets, self.pic, self.tol, self.kappa = nets, pic, tol, kappa

    def estimate(self, a0):
        p = [predict(n, self.pic, a0) for n in self.nets]
        mean = sum(p) / len(p)
        dis = rel_err(p[0], mean) if len(p) > 1 else np.full(a0.shape[0], np.inf)
        return mean, self.kappa * dis

    def calibrate(self, a0, aL, quantile=0.95):
        p = [predict(n, self.pic, a0) for n in self.nets]
        mean = sum(p) / len(p)
        dis = rel_err(p[0], mean)
        err = rel_err(mean, aL)
        self.kappa = float(np.quantile(err / np.maximum(dis, 1e-30), quantile))
        return err, dis

    def __call__(self, A0, z=SEGMENT_KM, precision="mixed"):
        """Fields after the segment for input fields A0 [count, n] (numpy complex)."""
        A0t = torch.as_tensor(A0, dtype=torch.complex128, device=self.pic.dev)
        scale = A0t.abs().amax(dim=1, keepdim=True)
        mean, est = self.estimate(A0t / scale)
        out = (self.pic.from_ip(mean, z) * scale).cpu().numpy()
        accept = est <= self.tol
        rej = np.nonzero(~accept)[0]
        if len(rej):
            out[rej], _ = propagate(A0[rej], z, precision)
        return out, accept, est
