"""``System`` container with the pyofss module protocol (pyofss/system.py:61-243).

A system holds a domain, a field and an ordered list of modules; ``run``
calls ``module(domain, field)`` in order and keeps each module's output field
under its name.  Any object with ``name`` and ``__call__(domain, field)``
(pulse generators, CUDA ``Fibre``s, the reference's lumped modules) plugs in.
"""

import numpy as np

from .domain import Domain


def field_save(field, filename="field_out"):
    np.savez_compressed(filename, field=field)


def field_load(filename="field_out"):
    if filename.endswith(".npz"):
        return np.load(filename)["field"]
    if filename.endswith(".npy"):
        return np.load(filename)
    try:
        return np.load(filename + ".npz")["field"]
    except OSError:
        return np.load(filename + ".npy")


class System:
    def __init__(self, domain=None, field=None):
        self.domain = Domain() if domain is None else domain
        self.modules = []
        self.fields = {}
        self.clear(remove_modules=True)
        if field is not None:
            self.field = field

    def clear(self, remove_modules=False):
        if self.domain.channels > 1:
            self.field = [np.zeros(self.domain.total_samples, complex)
                          for _ in range(self.domain.channels)]
        else:
            self.field = np.zeros(self.domain.total_samples, complex)
        self.fields = {}
        if remove_modules:
            self.modules = []

    def add(self, module):
        self.modules.append(module)

    def add_modules(self, modules):
        self.modules.extend(modules)

    def __getitem__(self, name):
        for m in self.modules:
            if m.name == name:
                return m
        return None

    def __setitem__(self, name, new_module):
        for i, m in enumerate(self.modules):
            if m.name == name:
                self.modules[i] = new_module
                return
        raise Exception("Tried to modify non-existing module in system")

    def run(self):
        for module in self.modules:
            self.field = module(self.domain, self.field)
            self.fields[module.name] = self.field
