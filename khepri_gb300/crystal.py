"""Drop-in ``Crystal`` for the reference's Crystal RCWA solve path, computed by libkhp on the GPU.

Method names, arguments, return values and error behaviour follow khepri/crystal.py:34-406:
``add_layer_uniform``, ``add_layer_pixmap``, ``add_pixmap_or_uniform``, ``add_layer``,
``set_device``, ``set_source``, ``solve``, ``poynting_flux_end``, ``fields_coords_xy``,
``fields_volume`` and the ``depth`` / ``zmax`` / ``solved`` / ``source_defined`` properties.

Differences a user may notice:
* ``S``/``Stot`` and the stacking matrices are torch complex128 CUDA tensors of the
  reference's shapes ([2, 2, n, n]); ``poynting_flux_end`` returns Python floats / numpy arrays.
* A layer solve that hits a singular pivot, a non-converged eigensolve or a non-finite value
  raises ``KhpError`` naming the condition instead of returning NaN silently.
* The convolution matrix, C^-1 and the Hx/Hy products of a pixmap are computed once per pixmap
  content, not on every ``solve`` (the reference rebuilds them, layer.py:156-158); the pixmap
  is still read at ``solve`` time, so in-place edits between solves are honoured.
* ``solve`` computes R and T of the source by the batched mixed-precision recursion
  (khp_solve_batched_mixed: FP32 eigensolve with FP64 refinement, FP64-refined stack
  equations; within ~1e-10 of complex128).  The S-matrices (``S``, ``Stot``, the stacking
  matrices) and what needs them (per-order powers, R and T of a source changed after ``solve``,
  fields) come from the FP64 layer-by-layer chain, built on first use from the same solve's
  inputs; their values are the reference's either way.
"""
from __future__ import annotations

import cmath
import math
from copy import copy
from types import SimpleNamespace

import numpy as np
import torch

from . import _capi, batch, engine
from .expansion import Expansion
from .engine import LayerSpec


class Layer:
    """Layer descriptors of the Layer API subset used by Crystal.add_layer (khepri/layer.py:63-143)."""

    def __init__(self, kind, eps, depth):
        self.kind, self.epsilon, self.depth = kind, eps, depth
        self.fields = False

    @classmethod
    def uniform(cls, expansion, epsilon, depth):
        """layer.py:113-120."""
        return cls("uniform", epsilon, depth)

    @classmethod
    def pixmap(cls, expansion, pixmap, depth):
        """layer.py:96-111."""
        return cls("pixmap", pixmap, depth)

    @classmethod
    def pixmap_or_uniform(cls, expansion, pixmap, depth):
        """layer.py:77-94: a uniform layer when every pixel holds the same value."""
        eps0 = np.asarray(pixmap).flatten()[0]
        if np.all(np.asarray(pixmap) == eps0):
            return cls.uniform(expansion, eps0, depth)
        return cls.pixmap(expansion, pixmap, depth)

    @classmethod
    def analytical(cls, expansion, islands_description, eps_host, depth):
        """layer.py:121-129: islands (Drawing.islands()) in a host medium, closed-form transforms."""
        return cls("pixmap", engine.AnalyticalMap(islands_description, eps_host), depth)

    @classmethod
    def half_infinite(cls, expansion, type, epsilon):
        """layer.py:132-143: "reflexion" (incidence side) or "transmission"; other types raise
        (the reference prints "ERROR")."""
        if type == "reflexion":
            return cls("inc", epsilon, 0)
        if type == "transmission":
            return cls("trn", epsilon, 0)
        raise ValueError(f"unknown half-space type {type!r}")

    def spec(self):
        """The layer as the engine's LayerSpec."""
        return LayerSpec(self.kind, self.epsilon, self.depth)


class _Built:
    """An attribute of a solved Crystal that comes from its S-matrix chain, built on first read."""

    def __set_name__(self, owner, name):
        self.slot = "_built_" + name

    def __get__(self, obj, owner=None):
        if obj is None:
            return self
        if obj._chain_pending:
            obj._build_chain()
        return obj.__dict__.get(self.slot)

    def __set__(self, obj, value):
        obj.__dict__[self.slot] = value


class Crystal:
    """GPU drop-in for khepri.crystal.Crystal (crystal.py:42-81; square, hexagonal or explicit
    lattices)."""

    S = _Built()
    Stot = _Built()
    stacking_matrices = _Built()
    stacking_reverse_matrices = _Built()
    _states = _Built()
    _fwd = _Built()
    _rev = _Built()
    _Stot_b = _Built()

    def __init__(self, pw, lattice="square", lattice_pitch=1, void=False, epsi=1, epse=1, device="cuda"):
        self.pw = tuple(pw)
        self.a = lattice_pitch
        self.void = void
        self.epsi = epsi
        self.epse = epse
        self.source = None
        self.lattice = engine.lattice_vectors(lattice, lattice_pitch)
        self.expansion = Expansion(self.pw, self.lattice)
        self._struct = engine.StructureGPU(self.pw, self.lattice, device)
        self.device = self._struct.device
        self.layers = dict()
        self._chain_pending = False
        self._solved = False
        self._rt = None
        self.stacking_matrices = list()
        self.stack_positions = []
        self.S = None

    # -- layers ----------------------------------------------------------------------------
    def add_layer_uniform(self, name, epsilon, depth):
        """crystal.py:97-103."""
        self.layers[name] = Layer("uniform", epsilon, depth)

    def add_pixmap_or_uniform(self, name, epsilon, depth):
        """crystal.py:104-111."""
        sample = np.asarray(epsilon).flatten()[0]
        if np.all(np.asarray(epsilon) == sample):
            self.add_layer_uniform(name, sample, depth)
        else:
            self.add_layer_pixmap(name, epsilon, depth)

    def add_layer_pixmap(self, name, epsilon, depth):
        """crystal.py:113-117 (the array is kept by reference, as layer.py:108 does)."""
        self.layers[name] = Layer("pixmap", epsilon, depth)

    def add_layer_analytical(self, name, epsilon, epsilon_host, depth):
        """crystal.py:119-123: ``epsilon`` is an islands description (Drawing.islands())."""
        self.layers[name] = Layer.analytical(None, epsilon, epsilon_host, depth)

    def add_layer(self, name, layer, extended=False):
        """crystal.py:125-129; extended layers belong to khepri_gb300.twisted."""
        if extended:
            raise NotImplementedError("extended (twisted) layers are not part of this GPU path")
        self.layers[name] = layer

    def set_device(self, layers_stack, fields_mask=False):
        """crystal.py:131-164."""
        self.device_stack = copy(layers_stack)
        self.global_stacking = []
        if not self.void:
            self.global_stacking.append("Sref")
        self.global_stacking.extend(layers_stack)
        if not self.void:
            self.global_stacking.append("Strans")
        required = set(self.global_stacking)
        if "Sref" in required and "Sref" not in self.layers:
            self.layers["Sref"] = Layer.half_infinite(None, "reflexion", self.epsi)
            self.layers["Sref"].fields = True
        if "Strans" in required and "Strans" not in self.layers:
            self.layers["Strans"] = Layer.half_infinite(None, "transmission", self.epse)
            self.layers["Strans"].fields = True
        fields_mask = [fields_mask] * len(layers_stack) if isinstance(fields_mask, bool) else fields_mask
        self.stack_retain_mask = [True] + list(fields_mask) + [True]
        for name, enabled in zip(self.global_stacking, self.stack_retain_mask):
            self.layers[name].fields |= enabled

    @property
    def depth(self):
        """crystal.py:166-170."""
        return sum(self.layers[name].depth for name in self.device_stack)

    @property
    def source_defined(self):
        """crystal.py:172-174."""
        return self.source is not None

    @property
    def solved(self):
        """crystal.py:176-178."""
        return self._solved

    @property
    def zmax(self):
        """crystal.py:398-400."""
        return self.stack_positions[-2]

    # -- source / solve --------------------------------------------------------------------
    def set_source(self, wavelength, te=1.0, tm=1.0, theta=0.0, phi=0.0, kp=None):
        """crystal.py:345-360."""
        self.source = SimpleNamespace(te=te, tm=tm, theta=theta, phi=phi, wavelength=wavelength)
        if kp is not None:
            self.kp = (kp[0], kp[1])
        else:
            self.kp = engine.compute_kplanar(self.epsi, wavelength, theta, phi)
        self.k0 = 2 * np.pi / wavelength
        self.kzi = np.conj(cmath.sqrt(self.k0 ** 2 * self.epsi - self.kp[0] ** 2 - self.kp[1] ** 2))

    def _problems(self):
        return engine.Problems.make([self.source.wavelength], [self.kp], self.source.te, self.source.tm, self.device)

    def _source_key(self):
        src = self.source
        return (src.wavelength, complex(src.te), complex(src.tm), complex(self.kp[0]), complex(self.kp[1]))

    def _fast_rt(self):
        """Whether R, T of the source can come from the batched recursion: both half-spaces are
        the crystal's own media and every device layer is homogeneous or patterned."""
        if self.void or self.global_stacking[:1] != ["Sref"] or self.global_stacking[-1:] != ["Strans"]:
            return False
        if self.layers["Sref"].kind != "inc" or self.layers["Strans"].kind != "trn":
            return False
        return all(self.layers[name].kind in ("uniform", "pixmap") for name in self.device_stack)

    def solve(self):
        """crystal.py:180-206: R and T of the source now (batched mixed-precision recursion);
        every distinct layer's S-matrix and the forward (and, when fields are retained, reverse)
        star-product chains when first read."""
        assert self.source_defined, "Call set_source before solving."
        prob = self._problems()
        layer_sizes = [self.layers[name].depth for name in self.global_stacking]
        self.stack_positions = list(np.cumsum(layer_sizes))
        self.stack_positions[-1] = np.inf
        if not self.void:
            self.stack_positions.insert(0, -np.inf)
        self._prob = prob
        self._chain_pending = True
        self._rt = None
        if self._fast_rt():
            specs = {name: self.layers[name].spec() for name in self.device_stack}
            specs["__inc__"] = LayerSpec("inc", self.epsi, 0.0)
            specs["__trn__"] = LayerSpec("trn", self.epse, 0.0)
            plan = batch.StackPlan(self._struct, specs, self.device_stack)
            status = torch.zeros(1, dtype=torch.int32, device=self.device)
            R, T = batch.solve_chunk_gamma(self._struct, plan, prob, status, self.epsi, self.epse, precision="mixed")
            word = int(status.item())
            if word:
                raise _capi.KhpError(f"solve: {_capi.decode_status(word)}")
            self._rt = (self._source_key(), float(R[0].item()), float(T[0].item()))
        else:
            self._build_chain()
        self._solved = True

    def _build_chain(self):
        """The layer S-matrices and star-product chains of the last solve (FP64 throughout)."""
        self._chain_pending = False
        prob = self._prob
        status = torch.zeros(1, dtype=torch.int32, device=self.device)
        specs = {name: self.layers[name].spec() for name in set(self.global_stacking)}
        keep = {name for name in specs if self.layers[name].fields}
        states = engine.solve_layers(self._struct, specs, self.global_stacking, prob, status, keep_modes=keep)
        want_fields = any(self.stack_retain_mask[1:-1])
        fwd, rev, Stot = engine.chain(states, self.global_stacking, self.stack_retain_mask, status,
                                      reverse=want_fields)
        word = int(status.item())
        if word:
            raise _capi.KhpError(f"solve: {_capi.decode_status(word)}")
        self._states = states
        self._fwd, self._rev = fwd, rev
        self.stacking_matrices = [None if s is None else s[0] for s in fwd]
        self.stacking_reverse_matrices = None if rev is None else [None if s is None else s[0] for s in rev]
        self.Stot = Stot[0]
        self.S = self.Stot
        self._Stot_b = Stot

    def poynting_flux_end(self, only_total=True):
        """crystal.py:363-396."""
        assert self.solved, "Call solve first"
        if only_total and self._rt is not None and self._rt[0] == self._source_key():
            return self._rt[1], self._rt[2]
        # the source as it is now (the reference reads self.source here, crystal.py:365-370)
        R, T, ro, to = engine.flux(self._struct, self._Stot_b, self._problems(), self.epsi, self.epse,
                                   orders=not only_total)
        if only_total:
            return float(R.item()), float(T.item())
        return (float(R.item()), ro[0].cpu().numpy()), (float(T.item()), to[0].cpu().numpy())

    # -- fields ------------------------------------------------------------------------------
    def get_source_as_field_vectors(self):
        """crystal.py:281-295: (E, H) source vectors, H = 0."""
        from .fields import incident_vector
        e = incident_vector(self.pw, self.source.te, self.source.tm, (self.kp[0], self.kp[1], self.kzi))
        return e, np.zeros_like(e)

    def fields_coords_xy(self, x, y, z, incident_fields=None, kp=None, return_fourier=False):
        """crystal.py:297-333: E, H at the (x, y) meshgrid for one depth z."""
        from . import fields
        return fields.fields_coords_xy(self, x, y, z, incident_fields, kp, return_fourier)

    def fields_volume(self, x, y, z, incident_fields=None):
        """crystal.py:335-343: E, H of shape [Nz, 3, X, Y]."""
        from . import fields
        return fields.fields_volume(self, x, y, z, incident_fields)


class Multilayer(Crystal):
    """1x1-harmonic Crystal (khepri/crystal.py:404-406)."""

    def __init__(self, epsi=1, epse=1, device="cuda"):
        super().__init__((1, 1), lattice="square", lattice_pitch=1, void=False, epsi=epsi, epse=epse, device=device)
