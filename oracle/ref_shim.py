"""Load the unmodified pyofss reference (pure Python) in a modern environment.

TEST INFRASTRUCTURE ONLY.  This module is used by ``tests/golden/make_golden.py``
and by the CPU tests that pin the oracle against the reference itself.  It is
never imported by the product package, by ``bench.py`` or on the GPU host
(the reference tree is not present there).

The reference targets an older numpy/scipy stack.  Without touching any file of
the reference, this shim:

* aliases the scipy names that newer scipy removed (``scipy.power``,
  ``scipy.log10``, ``scipy.exp``, ``scipy.sqrt``, ``scipy.log``,
  ``scipy.integrate.simps``) and ``collections.Iterable``;
* registers empty stand-ins for optional modules the reference imports at
  module level but never uses on the CPU propagation path (matplotlib,
  pyopencl, reikna, pynvml, unittest2), and, when pandas is absent, a
  ``read_csv`` for the numeric tables the Yb gain model reads;
* pre-registers ``pyofss`` as a package object with ``__path__`` so that
  ``pyofss/__init__.py`` (which pulls in the plotter and OpenCL modules) is not
  executed.

Runtime quirks of the reference that callers must work around:

* ``Stepper.adaptive_stepper`` reads ``storage.dir_spec`` at its end
  (pyofss/modules/stepper.py:365), an attribute ``Storage`` never defines;
  :func:`make_fibre` sets ``dir_spec = dir_temp = None`` on the instance.
* ``Stepper.__call__`` requires ``refrence_length`` (stepper.py:147);
  ``Fibre.__call__`` supplies it.
"""

import collections
import collections.abc
import importlib
import os
import sys
import types

import numpy as np

# The reference checkout: $PYOFSS_REFERENCE, else a directory named "reference" beside
# this repository's root (the repository and the pyofss checkout side by side).
REFERENCE_ROOT = os.environ.get(
    "PYOFSS_REFERENCE",
    os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference"))


class _Stub(types.ModuleType):
    """Module stand-in: any attribute is another stub (callable, subclassable)."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        sub = _Stub(f"{self.__name__}.{name}")
        setattr(self, name, sub)
        return sub

    def __call__(self, *args, **kwargs):
        return _Stub(self.__name__ + "()")

    def __mro_entries__(self, bases):
        return (object,)


class _Frame:
    """The part of a pandas DataFrame the reference uses: ``columns`` and column lookup."""

    def __init__(self, names, data):
        self.columns = names
        self._cols = {name: data[:, i] for i, name in enumerate(names)}

    def __getitem__(self, name):
        return self._cols[name]


def _mini_pandas():
    """``pandas.read_csv`` for the reference's numeric data tables, used by
    ``Amplifier2LevelModel.interpolate_sigma_s`` (pyofss/modules/amplifier.py:234-245).

    As pandas does with its default ``header="infer"``, the first line becomes the
    column names, so the first data row of a headerless table is not data; with
    ``header=None`` every line is data and the columns are 0, 1, ...  Values are
    parsed with Python's correctly rounded ``float``.
    """
    mod = types.ModuleType("pandas")

    def read_csv(path, delimiter=",", header="infer", **_):
        with open(path) as f:
            lines = [ln for ln in f.read().splitlines() if ln.strip()]
        names = None if header is None else lines[0].split(delimiter)
        rows = lines if header is None else lines[1:]
        data = np.array([[float(x) for x in r.split(delimiter)] for r in rows])
        return _Frame(list(range(data.shape[1])) if names is None else names, data)

    mod.read_csv = read_csv
    return mod


def available():
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "pyofss"))


_loaded = None


def load():
    """Import the reference's CPU propagation modules; return a namespace."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not available():
        raise RuntimeError(f"pyofss reference tree not found at {REFERENCE_ROOT}")
    sys.dont_write_bytecode = True

    import scipy
    import scipy.integrate

    for name in ("power", "log10", "exp", "sqrt", "log"):
        if not hasattr(scipy, name):
            setattr(scipy, name, getattr(np, name))
    if not hasattr(scipy.integrate, "simps"):
        scipy.integrate.simps = scipy.integrate.simpson
    if not hasattr(collections, "Iterable"):
        collections.Iterable = collections.abc.Iterable

    try:
        importlib.import_module("pandas")
    except Exception:
        sys.modules["pandas"] = _mini_pandas()
    for mod in ("matplotlib", "matplotlib.pyplot", "pyopencl",
                "pyopencl.array", "reikna", "reikna.cluda", "reikna.fft",
                "pynvml", "unittest2", "tqdm"):
        if mod not in sys.modules:
            try:
                importlib.import_module(mod)
            except Exception:
                sys.modules[mod] = _Stub(mod)

    if "pyofss" not in sys.modules:
        pkg = types.ModuleType("pyofss")
        pkg.__path__ = [os.path.join(REFERENCE_ROOT, "pyofss")]
        sys.modules["pyofss"] = pkg
        mods = types.ModuleType("pyofss.modules")
        mods.__path__ = [os.path.join(REFERENCE_ROOT, "pyofss", "modules")]
        sys.modules["pyofss.modules"] = mods

    ns = types.SimpleNamespace()
    ns.field = importlib.import_module("pyofss.field")
    ns.domain = importlib.import_module("pyofss.domain")
    ns.solver = importlib.import_module("pyofss.modules.solver")
    ns.stepper = importlib.import_module("pyofss.modules.stepper")
    ns.linearity = importlib.import_module("pyofss.modules.linearity")
    ns.nonlinearity = importlib.import_module("pyofss.modules.nonlinearity")
    ns.amplifier = importlib.import_module("pyofss.modules.amplifier")
    ns.fibre = importlib.import_module("pyofss.modules.fibre")
    ns.sech = importlib.import_module("pyofss.modules.sech")
    ns.gaussian = importlib.import_module("pyofss.modules.gaussian")
    ns.Domain = ns.domain.Domain
    ns.Fibre = ns.fibre.Fibre
    ns.Sech = ns.sech.Sech
    ns.Gaussian = ns.gaussian.Gaussian
    ns.Stepper = ns.stepper.Stepper
    _loaded = ns
    return ns


def make_fibre(**kwargs):
    """Build a reference ``Fibre`` with the adaptive-stepper end-of-run quirk patched."""
    ref = load()
    fib = ref.Fibre(**kwargs)
    fib.stepper.storage.dir_spec = None
    fib.stepper.storage.dir_temp = None
    # Storage.update_characts calls scipy find_peaks per trace; harmless, but
    # the characteristic lists are host analysis outside the propagation path.
    return fib


class StepLog:
    """Record every call (z, h) of one of the reference's step methods (``Solver.rk4ip``
    by default; static or bound, solver.py:81)."""

    def __init__(self, method="rk4ip"):
        self.method = method
        self.calls = []

    def __enter__(self):
        cls = load().solver.Solver
        self._raw = cls.__dict__[self.method]
        log = self.calls
        if isinstance(self._raw, staticmethod):
            orig = self._raw.__func__

            def logged(A, z, h, f):
                log.append((float(z), float(h)))
                return orig(A, z, h, f)

            setattr(cls, self.method, staticmethod(logged))
        else:
            orig = self._raw

            def logged_bound(obj, A, z, h, f):
                log.append((float(z), float(h)))
                return orig(obj, A, z, h, f)

            setattr(cls, self.method, logged_bound)
        return self

    def __exit__(self, *exc):
        setattr(load().solver.Solver, self.method, self._raw)
        return False
