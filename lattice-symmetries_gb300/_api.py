"""User-facing Python API mirroring the reference's python/lattice_symmetries/__init__.py.

``Symmetry``, ``Symmetries``, ``SpinBasis``, ``SpinfulFermionBasis``, ``SpinlessFermionBasis``,
``Expr`` and ``Operator`` keep the reference's names, constructor arguments and error behaviour
(RuntimeError from the library's error handler).  Underneath, this module plays the role of the
reference's Haskell host layer: it closes the symmetry group, writes the Benes masks and the
non-branching term tables into the C structs of include/ls_gb300.h, and calls the C ABI of
libls_gb300.so, whose kernels run on the GPU.

Additions with no counterpart in the reference: ``Operator.apply_device`` (device tensors, complex128,
several right-hand sides, adjoint), ``Basis.device_states`` / ``device_norms``.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_double, c_int, c_int64, c_uint8, c_uint64, c_void_p
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native as N
from ._expr import Expr, terms_to_arrays
from ._group import Symmetries, Symmetry

try:  # scipy is optional for the LinearOperator base class
    from scipy.sparse.linalg import LinearOperator as _LinearOperator
except Exception:  # pragma: no cover
    _LinearOperator = object
try:  # array namespace that recent scipy versions expect on every LinearOperator
    from scipy.sparse.linalg._interface import np_compat as _XP
except Exception:  # pragma: no cover
    _XP = np


def _u64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


class _DeviceArray:
    """Exposes a device pointer through __cuda_array_interface__ (read-only view)."""

    def __init__(self, ptr: int, shape, typestr: str, owner):
        self.__cuda_array_interface__ = {
            "shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False), "version": 3,
            "strides": None,
        }
        self._owner = owner


class Basis:
    """Common part of the three basis kinds (reference ``Basis``, __init__.py:147-330)."""

    def __init__(self, particle_type: int, number_sites: int, number_particles: int,
                 number_up: int, spin_inversion: int, symmetries: Optional[Symmetries]):
        lib = N.lib()
        self._lib = lib
        self._symmetries = symmetries if symmetries is not None else Symmetries([])
        self._keep = []
        self._c_kernels = N.ls_hs_basis_kernels()
        self._c = N.ls_hs_basis()
        c = self._c
        c.refcount = 1
        c.number_sites = number_sites
        c.number_particles = number_particles
        c.number_up = number_up
        c.particle_type = particle_type
        c.spin_inversion = spin_inversion
        has_perm = particle_type in (N.LS_HS_SPIN, N.LS_HS_SPINFUL_FERMION) and self._symmetries.order > 0
        c.requires_projection = bool(has_perm or spin_inversion != 0)
        c.state_index_is_identity = self._index_is_identity()
        c.kernels = ctypes.pointer(self._c_kernels)
        c.representatives = N.chpl_external_array(None, 0, None)
        self._orbit_data = None
        if has_perm:
            self._orbit_data = self._create_orbit_data()
            addr_si = N.fn_address("ls_hs_state_info_halide_kernel")
            addr_ir = N.fn_address("ls_hs_is_representative_halide_kernel")
            self._c_kernels.state_info_kernel = addr_si
            self._c_kernels.state_info_data = self._orbit_data
            self._c_kernels.is_representative_kernel = addr_ir
            self._c_kernels.is_representative_data = self._orbit_data

    # -- construction helpers ---------------------------------------------------------------------
    def _index_is_identity(self) -> bool:
        """Basis.hs:701-707."""
        raise NotImplementedError

    def _create_orbit_data(self):
        masks, shifts = self._symmetries.network()
        re, im = self._symmetries.characters
        masks = np.ascontiguousarray(masks, dtype=np.uint64)
        shifts = np.ascontiguousarray(shifts, dtype=np.uint64)
        g = N.ls_hs_permutation_group()
        g.refcount = 0
        g.number_bits = self._symmetries.number_bits
        g.number_shifts = int(masks.shape[0])
        g.number_masks = int(masks.shape[1]) if masks.ndim == 2 else 0
        g.masks = N.as_ptr(masks, c_uint64)
        g.shifts = N.as_ptr(shifts, c_uint64)
        g.eigvals_re = N.as_ptr(re, c_double)
        g.eigvals_im = N.as_ptr(im, c_double)
        if self._c.particle_type == N.LS_HS_SPINFUL_FERMION:
            ptr = self._lib.ls_gpu_create_fermionic_kernel_data(byref(g), int(self._c.number_sites))
        else:
            ptr = self._lib.ls_internal_create_halide_kernel_data(byref(g), int(self._c.spin_inversion))
        N.check()
        if not ptr:
            raise RuntimeError("could not create the orbit-scan data")
        return ptr

    def __del__(self):
        try:
            lib = self._lib
            k = self._c_kernels
            if k.state_index_data:
                lib.ls_hs_destroy_state_index_binary_search_kernel_data(k.state_index_data)
                k.state_index_data = None
            if self._orbit_data:
                lib.ls_internal_destroy_halide_kernel_data(self._orbit_data)
                self._orbit_data = None
            if self._c.representatives.elts and self._c.representatives.freer:
                lib.ls_hs_internal_destroy_external_array(byref(self._c.representatives))
                self._c.representatives = N.chpl_external_array(None, 0, None)
        except Exception:
            pass

    @property
    def _payload(self):
        return ctypes.pointer(self._c)

    # -- reference API ----------------------------------------------------------------------------
    @property
    def is_built(self) -> bool:
        return bool(self._c.representatives.elts)

    def check_is_built(self):
        if not self.is_built:
            raise ValueError("basis states have not been built yet; "
                             "if you wish to do so, use the basis.build() function")

    @property
    def min_state_estimate(self) -> int:
        return self._estimates()[0]

    @property
    def max_state_estimate(self) -> int:
        return self._estimates()[1]

    def _estimates(self) -> Tuple[int, int]:
        raise NotImplementedError

    def build(self, exact_norms: bool = False) -> None:
        """Generate the sorted list of representatives on the GPU (ls_hs_basis_build).

        exact_norms=False keeps the reference's membership rule (floating stabiliser sum > 0);
        exact_norms=True drops the states whose exact orbit norm is zero, which the floating rule
        can keep in complex sectors as rounding residue."""
        if not self.is_built:
            if self.number_bits > 64:
                raise RuntimeError("too many bits")
            lo, hi = self._estimates()
            previous = self._lib.ls_gpu_set_enumeration_rule(int(bool(exact_norms)))
            try:
                self._lib.ls_hs_build_representatives(self._payload, lo, hi)
            finally:
                self._lib.ls_gpu_set_enumeration_rule(previous)
            N.check()
        assert self.is_built

    @property
    def number_states(self) -> int:
        self.check_is_built()
        return int(self._c.representatives.num_elts)

    @property
    def states(self) -> np.ndarray:
        n = self.number_states
        if n == 0:
            return np.zeros(0, dtype=np.uint64)
        buf = (ctypes.c_uint64 * n).from_address(self._c.representatives.elts)
        arr = np.frombuffer(buf, dtype=np.uint64)
        arr.flags.writeable = False
        return arr

    @property
    def number_bits(self) -> int:
        return self._number_bits()

    def _number_bits(self) -> int:
        raise NotImplementedError

    @property
    def number_words(self) -> int:
        return (self.number_bits + 63) // 64

    @property
    def has_spin_inversion_symmetry(self) -> bool:
        return self._c.spin_inversion != 0

    @property
    def has_permutation_symmetries(self) -> bool:
        return self._orbit_data is not None

    @property
    def requires_projection(self) -> bool:
        return bool(self._c.requires_projection)

    @property
    def symmetries(self) -> Symmetries:
        return self._symmetries

    def state_info(self, x):
        """(representatives, characters, norms), __init__.py:256-296."""
        is_scalar = isinstance(x, (int, np.integer))
        x = np.array([x], dtype=np.uint64) if is_scalar else _u64(x)
        count = x.shape[0]
        if self.has_permutation_symmetries:
            betas = np.zeros_like(x)
            chars = np.zeros(count, dtype=np.complex128)
            norms = np.zeros(count, dtype=np.float64)
            if count > 0:
                self._lib.ls_hs_state_info(self._payload, count, N.as_ptr(x, c_uint64), 1,
                                           N.as_ptr(betas, c_uint64), 1,
                                           chars.ctypes.data_as(POINTER(c_double)),
                                           N.as_ptr(norms, c_double))
                N.check()
        elif self.has_spin_inversion_symmetry:
            mask = np.uint64((1 << self.number_bits) - 1)
            b = np.bitwise_xor(x, mask)
            when = b < x
            betas = np.where(when, b, x)
            chars = np.where(when, float(self._c.spin_inversion), 1.0).astype(np.complex128)
            norms = np.ones(count, dtype=np.float64)
        else:
            betas = x
            chars = np.ones(count, dtype=np.complex128)
            norms = np.ones(count, dtype=np.float64)
        if is_scalar:
            return (int(betas[0]), complex(chars[0]), float(norms[0]))
        return (betas, chars, norms)

    def is_representative(self, x):
        """(flags, raw norms) of ls_hs_is_representative."""
        x = _u64(np.atleast_1d(x))
        flags = np.zeros(x.shape[0], dtype=np.uint8)
        norms = np.zeros(x.shape[0], dtype=np.float64)
        if x.shape[0] > 0:
            self._lib.ls_hs_is_representative(self._payload, x.shape[0], N.as_ptr(x, c_uint64), 1,
                                              N.as_ptr(flags, c_uint8), N.as_ptr(norms, c_double))
            N.check()
        return flags, norms

    def index(self, x):
        """Index of basis states (-1 if absent), __init__.py:298-318."""
        x = np.asarray(x, dtype=np.uint64, order="C")
        is_scalar = x.ndim == 0
        if is_scalar:
            x = np.expand_dims(x, axis=0)
        x = np.ascontiguousarray(x)
        out = np.zeros(x.shape[0], dtype=np.int64)
        if x.shape[0] > 0:
            self.check_is_built()
            self._lib.ls_hs_state_index(self._payload, x.shape[0], N.as_ptr(x, c_uint64), 1,
                                        N.as_ptr(out, c_int64), 1)
            N.check()
        return int(out[0]) if is_scalar else out

    # -- GPU views (additive) ---------------------------------------------------------------------
    def _device_info(self):
        self.check_is_built()
        n = c_int64(0)
        reps = c_void_p(0)
        norms = c_void_p(0)
        rc = self._lib.ls_gpu_basis_info(self._payload, byref(n), byref(reps), byref(norms))
        N.check(rc, "ls_gpu_basis_info")
        return n.value, reps.value, norms.value

    def device_states(self):
        """Device array of representatives (a __cuda_array_interface__ view, uint64)."""
        n, reps, _ = self._device_info()
        return _DeviceArray(reps, (n,), "<u8", self)

    def device_norms(self):
        n, _, norms = self._device_info()
        return _DeviceArray(norms, (n,), "<f8", self)

    # -- persistence (the role of the reference's HDF5 basis files, MyHDF5.chpl:255-335) -------
    def json_object(self) -> dict:
        raise NotImplementedError

    def save(self, path: str) -> None:
        """Writes the basis definition and its representatives to `path` (numpy .npz), so that a
        large basis is enumerated once and loaded afterwards."""
        import json
        self.check_is_built()
        np.savez(path, representatives=np.asarray(self.states, dtype=np.uint64),
                 definition=np.array(json.dumps(self.json_object())))

    def _set_representatives(self, states: np.ndarray) -> None:
        """Installs externally stored representatives (ls_hs_unchecked_set_representatives): the
        array is kept by this object and indexed on the GPU."""
        if self.is_built:
            raise ValueError("representatives have already been set")
        states = np.ascontiguousarray(states, dtype=np.uint64)
        if len(states) > 1 and not np.all(states[1:] > states[:-1]):
            raise ValueError("representatives must be sorted and unique")
        self._loaded_states = states
        arr = N.chpl_external_array(states.ctypes.data if len(states) else None, len(states), None)
        self._lib.ls_hs_unchecked_set_representatives(self._payload, byref(arr), 22)
        N.check()


def basis_from_json(obj: dict) -> Basis:
    """The basis described by Basis.json_object() (not built)."""
    syms = obj.get("symmetries") or []
    symmetries = Symmetries([Symmetry(s["permutation"], s["sector"]) for s in syms]) if syms else None
    particle = obj["particle"]
    if particle == "spin-1/2":
        return SpinBasis(obj["number_spins"], obj.get("hamming_weight"), obj.get("spin_inversion"), symmetries)
    if particle == "spinful-fermion":
        occ = obj.get("number_particles")
        return SpinfulFermionBasis(obj["number_sites"], tuple(occ) if isinstance(occ, list) else occ, symmetries)
    if particle == "spinless-fermion":
        return SpinlessFermionBasis(obj["number_sites"], obj.get("number_particles"))
    raise ValueError("unknown particle type: {}".format(particle))


def load_basis(path: str) -> Basis:
    """A basis written by Basis.save, with its representatives installed (no enumeration)."""
    import json
    with np.load(path, allow_pickle=False) as f:
        basis = basis_from_json(json.loads(str(f["definition"])))
        basis._set_representatives(f["representatives"])
    return basis


def _popcount(x: int) -> int:
    return bin(x).count("1")


class SpinBasis(Basis):
    """Spin-1/2 basis (__init__.py:330-356, Basis.hs:321-345)."""

    def __init__(self, number_spins: int, hamming_weight: Optional[int] = None,
                 spin_inversion: Optional[int] = None, symmetries: Optional[Symmetries] = None):
        n = int(number_spins)
        if n <= 0:
            raise ValueError("invalid number of spins: {}".format(n))
        if hamming_weight is not None and (hamming_weight < 0 or hamming_weight > n):
            raise ValueError("invalid Hamming weight: {}".format(hamming_weight))
        if spin_inversion is not None and spin_inversion not in (-1, 1):
            raise ValueError("invalid spin inversion: {}".format(spin_inversion))
        if spin_inversion is not None and hamming_weight is None:
            hamming_weight = n // 2
        if spin_inversion is not None and n != 2 * hamming_weight:
            raise ValueError("invalid spin inversion: {} spins, but Hamming weight is {}".format(
                n, hamming_weight))
        if symmetries is not None and symmetries.order > 0 and symmetries.number_bits != n:
            raise ValueError("invalid symmetries")
        self.number_spins = n
        self.hamming_weight = hamming_weight
        super().__init__(N.LS_HS_SPIN, n, n, -1 if hamming_weight is None else int(hamming_weight),
                         0 if spin_inversion is None else int(spin_inversion), symmetries)

    def json_object(self) -> dict:
        inv = int(self._c.spin_inversion)
        return {"particle": "spin-1/2", "number_spins": self.number_spins, "hamming_weight": self.hamming_weight,
                "spin_inversion": inv if inv != 0 else None, "symmetries": self.symmetries.json_object()}

    def _index_is_identity(self) -> bool:
        return self.hamming_weight is None and self._c.spin_inversion == 0 and self._symmetries.order == 0

    def _number_bits(self) -> int:
        return self.number_spins

    def _estimates(self):
        """Basis.hs:734-774."""
        n, h = self.number_spins, self.hamming_weight
        if h is None:
            return 0, (1 << n) - 1
        lo = (1 << h) - 1
        hi = ((1 << h) - 1) << (n - h - (1 if self._c.spin_inversion != 0 else 0))
        return lo, hi

    @property
    def has_fixed_hamming_weight(self) -> bool:
        return self.hamming_weight is not None

    @property
    def spin_inversion(self) -> Optional[int]:
        i = self._c.spin_inversion
        return int(i) if i != 0 else None


class SpinlessFermionBasis(Basis):
    def __init__(self, number_sites: int, number_particles: Optional[int] = None):
        n = int(number_sites)
        if n <= 0:
            raise ValueError("invalid number of sites: {}".format(n))
        if number_particles is not None and (number_particles < 0 or number_particles > n):
            raise ValueError("invalid number of particles: {}".format(number_particles))
        self.number_sites = n
        self.number_particles = number_particles
        super().__init__(N.LS_HS_SPINLESS_FERMION, n,
                         -1 if number_particles is None else int(number_particles), -1, 0, None)

    def json_object(self) -> dict:
        return {"particle": "spinless-fermion", "number_sites": self.number_sites,
                "number_particles": self.number_particles}

    def _index_is_identity(self) -> bool:
        return self.number_particles is None

    def _number_bits(self) -> int:
        return self.number_sites

    def _estimates(self):
        n, p = self.number_sites, self.number_particles
        if p is None:
            return 0, (1 << n) - 1
        return (1 << p) - 1, ((1 << p) - 1) << (n - p)


class SpinfulFermionBasis(Basis):
    """Spinful fermions: bits [0, n) are the up spins, [n, 2n) the down spins (Basis.hs:621-628).

    ``symmetries`` (an addition: the reference has no fermionic lattice symmetries,
    Basis.hs:713-723) are site permutations; each acts on both spin species and on Fock states
    with the sign of the permutation of the occupied orbitals.  They need fixed (N_up, N_down)."""

    def __init__(self, number_sites: int, number_particles: Union[None, int, Tuple[int, int]] = None,
                 symmetries: Optional[Symmetries] = None):
        n = int(number_sites)
        if n <= 0:
            raise ValueError("invalid number of sites: {}".format(n))
        self.number_sites = n
        if number_particles is None:
            total, up = -1, -1
            self.occupation = None
        elif isinstance(number_particles, (tuple, list)):
            u, d = (int(v) for v in number_particles)
            if u < 0 or u > n or d < 0 or d > n:
                raise ValueError("invalid number of particles: {} up, {} down".format(u, d))
            total, up = u + d, u
            self.occupation = (u, d)
        else:
            p = int(number_particles)
            if p < 0 or p > 2 * n:
                raise ValueError("invalid number of particles: {}".format(p))
            total, up = p, -1
            self.occupation = p
        doubled = None
        if symmetries is not None and symmetries.order > 0:
            if symmetries.number_bits != n:
                raise ValueError("symmetries act on {} sites, the basis has {}".format(symmetries.number_bits, n))
            if not isinstance(self.occupation, tuple):
                raise ValueError("lattice symmetries of spinful fermions need fixed (N_up, N_down)")
            doubled = symmetries.doubled()
        self.site_symmetries = symmetries
        super().__init__(N.LS_HS_SPINFUL_FERMION, n, total, up, 0, doubled)

    def json_object(self) -> dict:
        occ = list(self.occupation) if isinstance(self.occupation, tuple) else self.occupation
        syms = self.site_symmetries.json_object() if self.site_symmetries is not None else []
        return {"particle": "spinful-fermion", "number_sites": self.number_sites, "number_particles": occ,
                "symmetries": syms}

    def _index_is_identity(self) -> bool:
        return self.occupation is None and (self.site_symmetries is None or self.site_symmetries.order == 0)

    def _number_bits(self) -> int:
        return 2 * self.number_sites

    def _estimates(self):
        n = self.number_sites
        if self.occupation is None:
            return 0, (1 << (2 * n)) - 1
        if isinstance(self.occupation, tuple):
            u, d = self.occupation
            lo = (((1 << d) - 1) << n) | ((1 << u) - 1)
            hi = ((((1 << d) - 1) << (n - d)) << n) | (((1 << u) - 1) << (n - u))
            return lo, hi
        p = self.occupation
        return (1 << p) - 1, ((1 << p) - 1) << (2 * n - p)


def split_terms(basis: Basis, expression: Expr):
    """(off-diagonal, diagonal) non-branching terms of `expression` on `basis` (Operator.hs:109-135)."""
    n_sites = getattr(basis, "number_sites", None) or getattr(basis, "number_spins")
    spinful = isinstance(basis, SpinfulFermionBasis)
    terms = expression.nonbranching_terms(n_sites, spinful=spinful)
    return [t for t in terms if t[4] != 0], [t for t in terms if t[4] == 0]


def _terms_struct(arrays, number_bits: int, keep: list):
    v, m, l, r, x, s = arrays
    n = len(v)
    if n == 0:
        return None
    v = np.ascontiguousarray(v, dtype=np.complex128)
    arrs = [np.ascontiguousarray(a, dtype=np.uint64) for a in (m, l, r, x, s)]
    keep.extend([v] + arrs)
    t = N.ls_hs_nonbranching_terms()
    t.number_terms = n
    t.number_bits = number_bits
    t.v = v.ctypes.data_as(POINTER(c_double))
    t.m, t.l, t.r, t.x, t.s = (a.ctypes.data_as(POINTER(c_uint64)) for a in arrs)
    keep.append(t)
    return t


class Operator(_LinearOperator):
    """A quantum operator on a basis (__init__.py:591-759): a scipy LinearOperator on float64
    vectors whose product runs on the GPU through ls_chpl_matrix_vector_product."""

    def __init__(self, basis: Basis, expression: Expr):
        if not isinstance(basis, Basis):
            raise TypeError("expected a 'Basis', but got '{}'".format(type(basis)))
        if not isinstance(expression, Expr):
            raise TypeError("expected an 'Expr', but got '{}'".format(type(expression)))
        off, diag = split_terms(basis, expression)
        self._setup(basis, expression, terms_to_arrays(off), terms_to_arrays(diag))

    @classmethod
    def _from_arrays(cls, basis: Basis, off_arrays, diag_arrays, expression: Optional[Expr] = None):
        """An operator from raw non-branching term arrays (v, m, l, r, x, s); the arrays are kept
        and read by the library on every call, so changing v in place re-parametrises it."""
        op = cls.__new__(cls)
        op._setup(basis, expression, off_arrays, diag_arrays)
        return op

    def _setup(self, basis, expression, off_arrays, diag_arrays):
        self._basis = basis
        self._expression = expression
        self._off_arrays = tuple(np.ascontiguousarray(a) for a in off_arrays)
        self._diag_arrays = tuple(np.ascontiguousarray(a) for a in diag_arrays)
        self._keep = []
        nb = basis.number_bits
        self._c_off = _terms_struct(self._off_arrays, nb, self._keep)
        self._c_diag = _terms_struct(self._diag_arrays, nb, self._keep)
        self._c = N.ls_hs_operator()
        self._c.refcount = 1
        self._c.basis = basis._payload
        self._c.off_diag_terms = ctypes.pointer(self._c_off) if self._c_off is not None else None
        self._c.diag_terms = ctypes.pointer(self._c_diag) if self._c_diag is not None else None
        self._lib = N.lib()
        # LinearOperator state (dtype and shape are properties here, resolved once the basis is
        # built, as in the reference's Operator)
        self._xp = _XP
        self.ndim = 2

    @property
    def _payload(self):
        return ctypes.pointer(self._c)

    def __del__(self):
        try:
            if getattr(self, "_c", None) is not None:
                self._lib.ls_gpu_release_operator(ctypes.pointer(self._c))
        except Exception:
            pass

    @property
    def basis(self) -> Basis:
        return self._basis

    @property
    def expression(self) -> Expr:
        return self._expression

    @property
    def number_off_diag_terms(self) -> int:
        return len(self._off_arrays[0])

    @property
    def number_diag_terms(self) -> int:
        return len(self._diag_arrays[0])

    def adjoint_operator(self) -> "Operator":
        return Operator(self._basis, self._expression.adjoint())

    def __add__(self, other):
        return Operator(self._basis, self._expression + other._expression)

    def __sub__(self, other):
        return Operator(self._basis, self._expression - other._expression)

    def scale(self, c) -> "Operator":
        return Operator(self._basis, self._expression.scale(c))

    def __rmul__(self, other):
        if np.isscalar(other):
            return self.scale(other)
        return NotImplemented

    def __matmul__(self, other):
        return self.apply_to_state_vector(other)

    def __repr__(self):
        return "<Operator defined on {}>".format(self._basis.__class__.__name__)

    def _check_basis_is_built(self, attribute):
        if not self._basis.is_built:
            raise AttributeError(
                "'Operator' object has no attribute '{}' (did you forget to build the basis?)".format(attribute))

    @property
    def dtype(self):
        self._check_basis_is_built("dtype")
        return np.dtype("float64")

    @property
    def shape(self):
        self._check_basis_is_built("shape")
        n = self._basis.number_states
        return (n, n)

    def apply_to_state_vector(self, vector: np.ndarray) -> np.ndarray:
        """y = H x for one float64 vector (ls_chpl_matrix_vector_product)."""
        self._check_basis_is_built("apply_to_state_vector")
        if vector.dtype != np.float64:
            raise TypeError("expected a NDArray[float64], but got {}[{}]".format(
                type(vector).__name__, type(vector.dtype)))
        x = np.ascontiguousarray(vector)
        out = np.empty_like(x)
        kernels = self._lib.ls_hs_internal_get_chpl_kernels().contents
        f = ctypes.CFUNCTYPE(None, POINTER(N.ls_hs_operator), ctypes.c_int, POINTER(c_double),
                             POINTER(c_double))(kernels.matrix_vector_product)
        f(self._payload, 1, N.as_ptr(x, c_double), N.as_ptr(out, c_double))
        N.check()
        return out

    def apply_to_state_vectors(self, vectors: np.ndarray) -> np.ndarray:
        """H applied to several real vectors [k, D] (host, float64) in one reference-facing call
        (ls_chpl_matrix_vector_product with num_vectors = k; one orbit scan for all k)."""
        self._check_basis_is_built("apply_to_state_vectors")
        X = np.ascontiguousarray(vectors, dtype=np.float64)
        if X.ndim != 2 or X.shape[1] != self._basis.number_states:
            raise ValueError("expected an array of shape [k, {}]".format(self._basis.number_states))
        Y = np.empty_like(X)
        self._lib.ls_chpl_matrix_vector_product(self._payload, X.shape[0], N.as_ptr(X, c_double),
                                                N.as_ptr(Y, c_double))
        N.check()
        return Y

    def _matvec(self, x):
        x = np.asarray(x)
        if x.ndim == 2:
            return np.stack([self.apply_to_state_vector(np.ascontiguousarray(x[:, i]))
                             for i in range(x.shape[1])], axis=1)
        return self.apply_to_state_vector(np.ascontiguousarray(x, dtype=np.float64))

    def apply_diag_to_basis_state(self, state: int) -> float:
        arr = np.array([state], dtype=np.uint64)
        coeffs = N.chpl_external_array()
        self._lib.ls_chpl_operator_apply_diag(self._payload, 1, N.as_ptr(arr, c_uint64), byref(coeffs), 0)
        N.check()
        value = float(ctypes.cast(coeffs.elts, POINTER(c_double))[0])
        self._lib.ls_hs_internal_destroy_external_array(byref(coeffs))
        return value

    def apply_off_diag_to_basis_state(self, state: int) -> List[Tuple[complex, int]]:
        arr = np.array([state], dtype=np.uint64)
        betas, coeffs, offsets = N.chpl_external_array(), N.chpl_external_array(), N.chpl_external_array()
        self._lib.ls_chpl_operator_apply_off_diag(self._payload, 1, N.as_ptr(arr, c_uint64), byref(betas),
                                                  byref(coeffs), byref(offsets), 0)
        N.check()
        count = int(ctypes.cast(offsets.elts, POINTER(ctypes.c_int64))[1])
        out = []
        for k in range(count):
            c = ctypes.cast(coeffs.elts, POINTER(c_double))
            b = ctypes.cast(betas.elts, POINTER(c_uint64))
            out.append((complex(c[2 * k], c[2 * k + 1]), int(b[k])))
        for a in (betas, coeffs, offsets):
            if a.elts:
                self._lib.ls_hs_internal_destroy_external_array(byref(a))
        return out

    # -- GPU (additive) ---------------------------------------------------------------------------
    def apply_device(self, x, out=None, adjoint: bool = False, stream=None, check: bool = True):
        """y = H x (or H^dagger x) on CUDA tensors: complex128 or float64, shape [D] or [D, k].

        Complex arithmetic is exact (complex characters and coefficients are kept); float64
        follows the reference's real-part semantics.  With check=False the call is stream-ordered
        and does not synchronise; errors are then reported by ``check_errors()``.
        """
        import torch

        self._check_basis_is_built("matvec")
        if not (isinstance(x, torch.Tensor) and x.is_cuda):
            raise TypeError("expected a CUDA tensor")
        if x.dtype not in (torch.complex128, torch.float64):
            raise TypeError("expected complex128 or float64, got {}".format(x.dtype))
        D = self._basis.number_states
        squeeze = x.dim() == 1
        X = x.reshape(D, 1) if squeeze else x
        if X.dim() != 2 or X.shape[0] != D:
            raise ValueError("expected a tensor of shape [{}] or [{}, k]".format(D, D))
        if X.stride(1) != 1:
            X = X.contiguous()
        k = X.shape[1]
        if out is None:
            Y = torch.empty((D, k), dtype=X.dtype, device=X.device)
        else:
            Y = out.reshape(D, k)
        if stream is None:
            stream = torch.cuda.current_stream(X.device).cuda_stream
        f = self._lib.ls_gpu_matvec_c128 if X.dtype == torch.complex128 else self._lib.ls_gpu_matvec_f64
        rc = f(self._payload, k, X.data_ptr(), X.stride(0), Y.data_ptr(), Y.stride(0), int(adjoint), stream)
        N.check(rc, "matvec")
        if check:
            N.check(self._lib.ls_gpu_check_errors(stream), "matvec")
        return Y.reshape(D) if squeeze else Y

    def apply_diag_batch(self, alphas):
        """Diagonal values of device basis states (uint64 / int64 CUDA tensor [B]) -> float64 [B]."""
        import torch
        a = alphas.contiguous()
        ys = torch.empty(a.shape[0], dtype=torch.float64, device=a.device)
        stream = torch.cuda.current_stream(a.device).cuda_stream
        N.check(self._lib.ls_gpu_operator_apply_diag(self._payload, a.shape[0], a.data_ptr(), ys.data_ptr(), stream),
                "apply_diag")
        return ys

    def apply_off_diag_batch(self, alphas):
        """Off-diagonal targets of device basis states: (betas int64 [nnz] holding uint64 bit
        patterns, coeffs complex128 [nnz], offsets int64 [B + 1]), as in the reference's
        ls_chpl_operator_apply_off_diag."""
        import torch
        a = alphas.contiguous()
        B, T = a.shape[0], max(self.number_off_diag_terms, 0)
        betas = torch.empty(max(B * T, 1), dtype=torch.int64, device=a.device)
        coeffs = torch.empty(max(B * T, 1), dtype=torch.complex128, device=a.device)
        offsets = torch.empty(B + 1, dtype=torch.int64, device=a.device)
        stream = torch.cuda.current_stream(a.device).cuda_stream
        N.check(self._lib.ls_gpu_operator_apply_off_diag(self._payload, B, a.data_ptr(), betas.data_ptr(),
                                                         coeffs.data_ptr(), offsets.data_ptr(), stream),
                "apply_off_diag")
        n = int(offsets[-1].item())
        return betas[:n], coeffs[:n], offsets

    def check_errors(self, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        N.check(self._lib.ls_gpu_check_errors(stream), "matvec")

    def autotune(self, k: int = 1):
        """Times the GPU matvec over (threads per block, grid waves) and, for k >= 8, the
        right-hand-side tile, and installs the fastest.  Returns (threads, waves, milliseconds)."""
        th, wv, ms = ctypes.c_int(0), ctypes.c_int(0), c_double(0.0)
        N.check(self._lib.ls_gpu_autotune_matvec(self._payload, int(k), byref(th), byref(wv), byref(ms)),
                "autotune")
        return th.value, wv.value, ms.value

    _ARITHMETIC = {"fp64": 0, "auto": 1, "pairs": 2}

    @staticmethod
    def block_arithmetic(mode: Optional[str] = None) -> str:
        """Arithmetic of complex blocks of 8 or 16 right-hand sides: "fp64" (default), "auto"
        (FP32-pair multiply-adds from an FP64 coefficient and a prescaled pair copy of x for
        groups of at most 64 elements, where FP64 bounds the kernel; each output within about
        2^-45 times the sum of its terms' magnitudes, ~1e-14 relative L2 to the FP64 form) or
        "pairs" (pairs for every group).  Sets it when `mode` is given; returns the mode in force."""
        lib = N.lib()
        codes = Operator._ARITHMETIC
        if mode is not None:
            if mode not in codes:
                raise ValueError("block arithmetic is 'auto', 'pairs' or 'fp64'")
            N.check(lib.ls_gpu_set_block_arithmetic(codes[mode]), "block arithmetic")
        cur = lib.ls_gpu_get_block_arithmetic()
        return {v: k for k, v in codes.items()}[cur]

    @staticmethod
    def launch_config():
        """(threads per block, grid waves, right-hand-side tile) used by the matvec kernels."""
        th, wv, tile = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        N.lib().ls_gpu_get_matvec_config(byref(th), byref(wv), byref(tile))
        return th.value, wv.value, tile.value

    def count_nonzeros(self) -> int:
        """Off-diagonal matrix elements of H in this basis (generated targets found in the basis)."""
        n = c_int64(0)
        N.check(self._lib.ls_gpu_count_nonzeros(self._payload, byref(n)), "count_nonzeros")
        return int(n.value)

    def kernel_info(self):
        """(form, slots_per_lane) of the matvec kernel: form "packed", "fallback" or "plain"."""
        form, slots = c_int(0), c_int(0)
        N.check(self._lib.ls_gpu_matvec_kernel_info(self._payload, byref(form), byref(slots)), "kernel_info")
        return ("plain", "fallback", "packed")[form.value], int(slots.value)


def load_library():
    return N.lib()


def set_tracing(on: bool = True) -> None:
    """Per-stage timing of the library (NVTX ranges and CUDA-event pairs around enumeration,
    index build, orbit norms, prescale and matvec kernels, batched and coupling kernels and the
    eigensolver's dense products); off by default.  Do not switch it on during a CUDA-graph
    capture."""
    N.lib().ls_gpu_set_tracing(int(bool(on)))


def stage_times(reset: bool = True, host: bool = False) -> dict:
    """{stage: (launches, total milliseconds)} of the traced stages since the last reset (waits
    for the traced work to finish): GPU time between the stage's events, or with host=True the
    wall time the calling thread spent inside the stage."""
    lib = N.lib()
    n = lib.ls_gpu_trace_report(None, 0, 0)
    buf = ctypes.create_string_buffer(n + 1)
    lib.ls_gpu_trace_report(ctypes.addressof(buf), n + 1, int(bool(reset)))
    out = {}
    for line in buf.value.decode().splitlines():
        name, count, ms, host_ms = line.split()
        out[name] = (int(count), float(host_ms if host else ms))
    return out


class SectorBatch:
    """H_s X_s for many symmetry sectors s at once (the batched form of Operator.apply_device).

    ``operators`` holds one Operator per sector, each on its own built basis (typically the same
    Hamiltonian in all momentum / spin-inversion sectors of one group).  The batch owns two
    zero-padded complex128 tensors ``X`` and ``Y`` of shape [n_sectors, D_max, k]; sector s uses
    the rows [0, D_s) of ``X[s]`` and ``Y[s]`` (``x(s)``, ``y(s)`` are those views) and padding rows
    stay zero (D_max is rounded up to a multiple of 256).  ``run()`` computes Y = H X (or H^dagger X) with one persistent kernel launch per
    chunk of up to 16 right-hand sides over the rows of all sectors (``batched`` says whether the
    sectors could share one launch); ``capture()`` records that launch in a CUDA graph and
    ``replay()`` re-launches it.  No reference counterpart: the reference applies one operator to
    one real vector per call (DistributedMatrixVector.chpl:1096-1097).
    """

    def __init__(self, operators: List["Operator"], k: int = 1, adjoint: bool = False, device=None):
        import torch

        if len(operators) == 0:
            raise ValueError("need at least one operator")
        for op in operators:
            op._check_basis_is_built("SectorBatch")
        self._ops = list(operators)
        self._lib = N.lib()
        self.k = int(k)
        self.adjoint = bool(adjoint)
        self.sizes = [op.basis.number_states for op in operators]
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        d_max = (max(max(self.sizes), 1) + 255) // 256 * 256  # row blocks of 256 for Gram products
        self.X = torch.zeros((len(operators), d_max, self.k), dtype=torch.complex128, device=self.device)
        self.Y = torch.zeros_like(self.X)
        n = len(operators)
        ops_arr = (POINTER(N.ls_hs_operator) * n)(*[op._payload for op in operators])
        xs = (c_void_p * n)(*[self.X[s].data_ptr() for s in range(n)])
        ys = (c_void_p * n)(*[self.Y[s].data_ptr() for s in range(n)])
        plan = c_void_p(0)
        with torch.cuda.device(self.device):
            rc = self._lib.ls_gpu_sector_plan_create(n, ops_arr, self.k, xs, self.k, ys, self.k,
                                                     int(self.adjoint), byref(plan))
        N.check(rc, "sector plan")
        self._plan = plan
        self.batched = bool(self._lib.ls_gpu_sector_plan_is_batched(plan))
        self._graph = None

    def __del__(self):
        try:
            if getattr(self, "_plan", None) is not None and self._plan.value:
                self._lib.ls_gpu_sector_plan_destroy(self._plan)
                self._plan = None
        except Exception:
            pass

    @property
    def number_sectors(self) -> int:
        return len(self._ops)

    def x(self, s: int):
        return self.X[s, : self.sizes[s]]

    def y(self, s: int):
        return self.Y[s, : self.sizes[s]]

    def run(self, stream=None, check: bool = False):
        """Enqueues Y = H X on `stream` (default: torch's current stream); check=True synchronises
        and raises on a generated state outside its basis."""
        import torch

        if stream is None:
            stream = torch.cuda.current_stream(self.device).cuda_stream
        N.check(self._lib.ls_gpu_sector_plan_run(self._plan, stream), "sector matvec")
        if check:
            N.check(self._lib.ls_gpu_check_errors(stream), "sector matvec")
        return self.Y

    def autotune(self, stream=None) -> dict:
        """Times the batched form (one launch over all sectors) against one launch per sector and
        keeps the faster (recapture afterwards: a recorded graph keeps the form it recorded).
        Returns {"batched": bool, "ms_batched": t, "ms_per_sector": t}."""
        import torch

        if stream is None:
            stream = torch.cuda.current_stream(self.device).cuda_stream
        b, tb, tp = ctypes.c_int(0), c_double(0.0), c_double(0.0)
        N.check(self._lib.ls_gpu_sector_plan_autotune(self._plan, stream, byref(b), byref(tb), byref(tp)),
                "sector plan autotune")
        self.batched = bool(b.value)
        self._graph = None
        return {"batched": self.batched, "ms_batched": tb.value, "ms_per_sector": tp.value}

    def set_batched(self, batched: bool) -> None:
        """Forces the form: one launch over all sectors (True) or one launch per sector."""
        N.check(self._lib.ls_gpu_sector_plan_set_batched(self._plan, int(bool(batched))), "sector plan form")
        self.batched = bool(batched)
        self._graph = None

    def capture(self):
        """Records run() in a CUDA graph (after one uncaptured run that uploads every table)."""
        import torch

        self.run(check=True)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run(stream=s.cuda_stream)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()
        return self.Y

    def check_errors(self):
        import torch
        N.check(self._lib.ls_gpu_check_errors(torch.cuda.current_stream(self.device).cuda_stream), "sector matvec")
