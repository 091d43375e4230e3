"""Operator expressions and their non-branching term tables (host side).

An expression is a sum of scaled products of generators.  The GPU kernels consume the
non-branching representation of every product: a tuple ``(v, m, l, r, x, s)`` such that

    T |alpha> = v * [alpha & m == r] * (-1)^popcount(alpha & s) * |alpha ^ x>

(haskell/src/LatticeSymmetries/NonbranchingTerm.hs:17-33, arXiv:2203.04158 App. A).

* generator tuples: Generator.hs:229-247 (spins: 1, sigma^z, sigma^+, sigma^-; fermions:
  1, n, c^dagger, c with the Jordan-Wigner string on the lower bits);
* the product of two tuples: NonbranchingTerm.hs:43-58;
* primitive operators: sigma^x = sigma^+ + sigma^-, sigma^y = -i sigma^+ + i sigma^-,
  S = sigma/2 (Expr.hs:321-334);
* coefficients are exact rationals, converted to float64 once when the table is written
  (Operator.hs:124-131), so that terms which cancel symbolically (e.g. sigma^+ sigma^+ in
  sigma^x sigma^x + sigma^y sigma^y) cancel exactly;
* spinful sites flatten as (up, k) -> k and (down, k) -> n + k (Basis.hs:621-628);
* diagonal terms are those with x == 0 (NonbranchingTerm.hs:71-72, Operator.hs:152).

The text syntax follows the reference parser (Parser.hs:74-160): sums of optionally scaled
products, parentheses, sigma/S with a superscript x y z + - and a subscript site, and
c-dagger, c, n with a subscript site and an optional spin arrow.
"""

from __future__ import annotations

import re as _re
from fractions import Fraction
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np


class CQ:
    """Exact complex rational a + b i."""

    __slots__ = ("re", "im")

    def __init__(self, re=0, im=0):
        self.re = re if isinstance(re, Fraction) else Fraction(re)
        self.im = im if isinstance(im, Fraction) else Fraction(im)

    @staticmethod
    def of(z) -> "CQ":
        if isinstance(z, CQ):
            return z
        if isinstance(z, complex):
            return CQ(Fraction(z.real), Fraction(z.imag))
        if isinstance(z, (int, Fraction)):
            return CQ(Fraction(z), 0)
        if isinstance(z, (float, np.floating)):
            return CQ(Fraction(float(z)), 0)
        if isinstance(z, np.complexfloating):
            return CQ(Fraction(float(z.real)), Fraction(float(z.imag)))
        raise TypeError("invalid coefficient: {!r}".format(z))

    def __add__(self, o):
        o = CQ.of(o)
        return CQ(self.re + o.re, self.im + o.im)

    def __neg__(self):
        return CQ(-self.re, -self.im)

    def __sub__(self, o):
        return self + (-CQ.of(o))

    def __mul__(self, o):
        o = CQ.of(o)
        return CQ(self.re * o.re - self.im * o.im, self.re * o.im + self.im * o.re)

    def conj(self):
        return CQ(self.re, -self.im)

    def is_zero(self):
        return self.re == 0 and self.im == 0

    def __eq__(self, o):
        o = CQ.of(o)
        return self.re == o.re and self.im == o.im

    def __hash__(self):
        return hash((self.re, self.im))

    def to_complex(self) -> complex:
        return complex(float(self.re), float(self.im))

    def __repr__(self):
        return "CQ({}, {})".format(self.re, self.im)


# Non-branching tuples: (v: CQ, m, l, r, x, s) with Python ints as bit masks.
NBT = Tuple[CQ, int, int, int, int, int]


def nbt_compose(a: NBT, b: NBT) -> NBT:
    """Operator product a * b (b acts first), following NonbranchingTerm.hs:43-58.

    Masks m, l, r, x, s compose as in the reference.  The constant sign is the parity of the
    Jordan-Wigner strings evaluated on the fixed bits: b sees the input pattern r, a sees
    r ^ x_b, so p = popcount((r & s_b) ^ ((r ^ x_b) & s_a)).  The reference writes
    z = (r & s_b) ^ x_b in place of r ^ x_b; the two agree whenever r & ~s_b & s_a has even
    popcount, which holds for the normal-ordered products its algebra produces.  Products here
    are composed in the order written, so the general form is used.
    """
    va, ma, la, ra, _xa, sa = a
    vb, mb, lb, rb, xb, sb = b
    if ((ra ^ lb) & ma & mb) != 0:
        v = CQ(0)
    else:
        v = None
    m = ma | mb
    r = rb | (ra & ~mb)
    l = la | (lb & ~ma)
    x = l ^ r
    s = (sa ^ sb) & ~m
    p = bin((r & sb) ^ ((r ^ xb) & sa)).count("1")
    if v is None:
        v = va * vb
        if p % 2 == 1:
            v = -v
    return (v, m, l, r, x, s)


def nbt_adjoint(t: NBT) -> NBT:
    """T^dagger: conj(v) (-1)^popcount(x & s), l and r exchanged."""
    v, m, l, r, x, s = t
    v = v.conj()
    if bin(x & s).count("1") % 2 == 1:
        v = -v
    return (v, m, r, l, x, s)


# Generator kinds
SPIN_ID, SPIN_Z, SPIN_PLUS, SPIN_MINUS = "1", "z", "+", "-"
FERMION_ID, FERMION_N, FERMION_CREATE, FERMION_ANNIHILATE = "f1", "n", "c+", "c"

_ADJOINT_GEN = {SPIN_ID: SPIN_ID, SPIN_Z: SPIN_Z, SPIN_PLUS: SPIN_MINUS, SPIN_MINUS: SPIN_PLUS,
                FERMION_ID: FERMION_ID, FERMION_N: FERMION_N,
                FERMION_CREATE: FERMION_ANNIHILATE, FERMION_ANNIHILATE: FERMION_CREATE}


def generator_nbt(kind: str, i: int) -> NBT:
    """Generator.hs:229-247."""
    b = 1 << i
    if kind == SPIN_ID or kind == FERMION_ID:
        return (CQ(1), 0, 0, 0, 0, 0)
    if kind == SPIN_Z:
        return (CQ(-1), 0, 0, 0, 0, b)
    if kind == SPIN_PLUS:
        return (CQ(1), b, b, 0, b, 0)
    if kind == SPIN_MINUS:
        return (CQ(1), b, 0, b, b, 0)
    if kind == FERMION_N:
        return (CQ(1), b, b, b, 0, 0)
    if kind == FERMION_CREATE:
        return (CQ(1), b, b, 0, b, b - 1)
    if kind == FERMION_ANNIHILATE:
        return (CQ(1), b, 0, b, b, b - 1)
    raise ValueError("unknown generator: {}".format(kind))


# A site is an int (spins, spinless fermions) or a (spin, site) pair with spin 0 = up, 1 = down.
Product = Tuple[Tuple[str, object], ...]

_SPIN_KINDS = {SPIN_ID, SPIN_Z, SPIN_PLUS, SPIN_MINUS}


class Expr:
    """A polynomial in spin or fermion generators with exact complex-rational coefficients.

    ``Expr("2 (σ⁺₀ σ⁻₁ + σ⁺₁ σ⁻₀) + σᶻ₀ σᶻ₁", sites=[(0, 1), (1, 2)])`` replicates the
    expression over every tuple in ``sites`` (the reference's ``sites`` key,
    Expr.hs:372-383) and sums the copies.
    """

    def __init__(self, expression=None, sites: Optional[Sequence[Sequence[int]]] = None,
                 particle: Optional[str] = None):
        self.terms: List[Tuple[CQ, Product]] = []
        self.particle = particle
        if expression is None or (isinstance(expression, str) and expression.strip() == ""):
            return
        if isinstance(expression, str):
            parsed = _Parser(expression).parse()
            self.terms = parsed.terms
            self.particle = parsed.particle
        elif isinstance(expression, list):
            self.terms = list(expression)
        else:
            raise TypeError("invalid expression: {!r}".format(expression))
        if sites is not None:
            total = Expr(particle=self.particle)
            for tup in sites:
                mapping = {k: int(v) for k, v in enumerate(tup)}
                total = total + self.replace_indices(mapping)
            self.terms = total.terms

    # -- algebra ---------------------------------------------------------------------------------
    def _new(self, terms, other=None):
        e = Expr(particle=self.particle or (other.particle if other is not None else None))
        e.terms = terms
        return e

    def __add__(self, other: "Expr") -> "Expr":
        if not isinstance(other, Expr):
            return NotImplemented
        return self._new(self.terms + other.terms, other)

    def __sub__(self, other: "Expr") -> "Expr":
        if not isinstance(other, Expr):
            return NotImplemented
        return self + other.scale(-1)

    def __neg__(self):
        return self.scale(-1)

    def scale(self, c) -> "Expr":
        c = CQ.of(c)
        return self._new([(c * v, p) for v, p in self.terms])

    def __mul__(self, other):
        if isinstance(other, Expr):
            return self._new([(va * vb, pa + pb) for va, pa in self.terms for vb, pb in other.terms],
                             other)
        if np.isscalar(other):
            return self.scale(other)
        return NotImplemented

    def __rmul__(self, other):
        if np.isscalar(other):
            return self.scale(other)
        return NotImplemented

    def adjoint(self) -> "Expr":
        return self._new([(v.conj(), tuple((_ADJOINT_GEN[k], i) for k, i in reversed(p)))
                          for v, p in self.terms])

    def replace_indices(self, mapping) -> "Expr":
        """Relabel sites: ``{old: new}`` for site indices, or ``{(spin, old): (spin, new)}``."""
        def f(i):
            if isinstance(i, tuple):
                if i in mapping:
                    return tuple(mapping[i])
                return (i[0], mapping.get(i[1], i[1]))
            return mapping.get(i, i)
        return self._new([(v, tuple((k, f(i)) for k, i in p)) for v, p in self.terms])

    def __eq__(self, other):
        if not isinstance(other, Expr):
            return NotImplemented
        n = 1 + max(self._max_flat_index(), other._max_flat_index())
        a = self.nonbranching_terms(n)
        b = other.nonbranching_terms(n)
        return sorted(a, key=_nbt_key) == sorted(b, key=_nbt_key)

    def __hash__(self):
        return id(self)

    def _max_flat_index(self):
        m = -1
        for _, p in self.terms:
            for _, i in p:
                m = max(m, i[1] if isinstance(i, tuple) else i)
        return m

    # -- lowering -------------------------------------------------------------------------------
    def nonbranching_terms(self, number_sites: int, spinful: Optional[bool] = None) -> List[NBT]:
        """Merged non-branching tuples with non-zero coefficients, in first-appearance order."""
        if spinful is None:
            spinful = self.particle == "spinful-fermion"
        acc: Dict[Tuple[int, int, int, int, int], CQ] = {}
        order: List[Tuple[int, int, int, int, int]] = []
        for v, p in self.terms:
            t: NBT = (v, 0, 0, 0, 0, 0)
            for kind, site in p:
                if isinstance(site, tuple):
                    spin, k = site
                    flat = k + (number_sites if spin == 1 else 0)
                else:
                    flat = site
                    if spinful:
                        raise ValueError("spinful fermion operators need a spin index")
                t = nbt_compose(t, generator_nbt(kind, flat))
                if t[0].is_zero():
                    break
            if t[0].is_zero():
                continue
            key = t[1:]
            if key in acc:
                acc[key] = acc[key] + t[0]
            else:
                acc[key] = t[0]
                order.append(key)
        return [(acc[k],) + k for k in order if not acc[k].is_zero()]

    def __str__(self):
        parts = []
        for v, p in self.terms:
            parts.append("({}) {}".format(v.to_complex(), " ".join(_gen_str(k, i) for k, i in p)))
        return " + ".join(parts) if parts else "0"

    __repr__ = __str__


def _nbt_key(t: NBT):
    return (t[1:], t[0].re, t[0].im)


_SUP = {"ˣ": "x", "ʸ": "y", "ᶻ": "z", "⁺": "+", "⁻": "-"}
_SUB = {c: str(i) for i, c in enumerate("₀₁₂₃₄₅₆₇₈₉")}


def _gen_str(kind, i):
    names = {SPIN_Z: "σᶻ", SPIN_PLUS: "σ⁺", SPIN_MINUS: "σ⁻", SPIN_ID: "1", FERMION_ID: "1",
             FERMION_N: "n", FERMION_CREATE: "c†", FERMION_ANNIHILATE: "c"}
    if isinstance(i, tuple):
        return "{}{}{}".format(names[kind], i[1], "↑" if i[0] == 0 else "↓")
    return "{}{}".format(names[kind], i)


class _Parser:
    """Recursive-descent parser for the reference's expression syntax (Parser.hs:74-160)."""

    _number = _re.compile(r"[0-9]+(\.[0-9]*)?([eE][-+]?[0-9]+)?|\.[0-9]+([eE][-+]?[0-9]+)?")

    def __init__(self, text: str):
        self.s = text
        self.i = 0
        self.particle: Optional[str] = None

    def parse(self) -> Expr:
        e = self.p_sum()
        self.ws()
        if self.i != len(self.s):
            raise ValueError("could not parse expression at position {}: {!r}".format(
                self.i, self.s[self.i:]))
        e.particle = self.particle
        return e

    def ws(self):
        while self.i < len(self.s) and self.s[self.i].isspace():
            self.i += 1

    def peek(self):
        self.ws()
        return self.s[self.i] if self.i < len(self.s) else ""

    def p_sum(self) -> Expr:
        total = Expr()
        while True:
            c = self.peek()
            if c == "" or c == ")":
                break
            sign = 1
            if c in "+-":
                sign = -1 if c == "-" else 1
                self.i += 1
                if self.peek() in ("", ")", "+", "-"):
                    raise ValueError("dangling sign in expression")
            term = self.p_scaled()
            total = total + (term.scale(sign) if sign != 1 else term)
        return total

    def p_scaled(self) -> Expr:
        coeff = CQ(1)
        m = self._number.match(self.s, self.i) if self.peek() else None
        if m:
            coeff = CQ.of(float(m.group(0)))
            self.i = m.end()
            self.ws()
            if self.s.startswith("im", self.i) or self.s.startswith("ⅈ", self.i):
                coeff = CQ(0, coeff.re)
                self.i += 2 if self.s.startswith("im", self.i) else 1
        factors = []
        while True:
            c = self.peek()
            if c == "" or c in "+-)":
                break
            if c in "×*":
                self.i += 1
                continue
            if c == "(":
                self.i += 1
                inner = self.p_sum()
                if self.peek() != ")":
                    raise ValueError("missing ')' in expression")
                self.i += 1
                factors.append(inner)
            else:
                factors.append(self.p_primitive())
        if not factors:
            e = Expr([(CQ(1), ())])
        else:
            e = factors[0]
            for f in factors[1:]:
                e = e * f
        return e.scale(coeff)

    def p_subscript(self) -> int:
        digits = ""
        while self.i < len(self.s) and self.s[self.i] in _SUB:
            digits += _SUB[self.s[self.i]]
            self.i += 1
        if not digits:
            if self.i < len(self.s) and self.s[self.i] == "_":
                self.i += 1
            while self.i < len(self.s) and self.s[self.i].isdigit():
                digits += self.s[self.i]
                self.i += 1
        if not digits:
            raise ValueError("expected a site index at position {}".format(self.i))
        return int(digits)

    def p_primitive(self) -> Expr:
        s, i = self.s, self.i
        if s[i] in "σS":
            scale = Fraction(1, 2) if s[i] == "S" else Fraction(1)
            self.i += 1
            c = s[self.i] if self.i < len(s) else ""
            if c == "^":
                self.i += 1
                c = s[self.i]
            kind = _SUP.get(c, c if c in "xyz+-" else None)
            if kind is None:
                raise ValueError("expected a spin operator superscript at position {}".format(self.i))
            self.i += 1
            site = self.p_subscript()
            self._set_particle("spin-1/2")
            if kind == "x":
                terms = [(CQ(scale), ((SPIN_PLUS, site),)), (CQ(scale), ((SPIN_MINUS, site),))]
            elif kind == "y":
                terms = [(CQ(0, -scale), ((SPIN_PLUS, site),)), (CQ(0, scale), ((SPIN_MINUS, site),))]
            elif kind == "z":
                terms = [(CQ(scale), ((SPIN_Z, site),))]
            elif kind == "+":
                terms = [(CQ(scale), ((SPIN_PLUS, site),))]
            else:
                terms = [(CQ(scale), ((SPIN_MINUS, site),))]
            return Expr(terms)
        if s.startswith("c†", i):
            kind = FERMION_CREATE
            self.i += 2
        elif s[i] == "c":
            kind = FERMION_ANNIHILATE
            self.i += 1
        elif s[i] == "n":
            kind = FERMION_N
            self.i += 1
        else:
            raise ValueError("unexpected character {!r} at position {}".format(s[i], i))
        spin = None
        if self.i < len(s) and s[self.i] in "↑↓":  # the spin label may precede the site
            spin = 0 if s[self.i] == "↑" else 1
            self.i += 1
        site = self.p_subscript()
        if spin is None and self.i < len(s) and s[self.i] in "↑↓":
            spin = 0 if s[self.i] == "↑" else 1
            self.i += 1
        if spin is None:
            self._set_particle("spinless-fermion")
            return Expr([(CQ(1), ((kind, site),))])
        self._set_particle("spinful-fermion")
        return Expr([(CQ(1), ((kind, (spin, site)),))])

    def _set_particle(self, p):
        if self.particle is not None and self.particle != p:
            raise ValueError("expression mixes {} and {} operators".format(self.particle, p))
        self.particle = p


def terms_to_arrays(terms: Sequence[NBT]):
    """Float64/uint64 arrays (v as complex128, m, l, r, x, s) of a term list (Operator.hs:109-135)."""
    n = len(terms)
    v = np.zeros(n, dtype=np.complex128)
    arrs = [np.zeros(n, dtype=np.uint64) for _ in range(5)]
    for k, t in enumerate(terms):
        v[k] = t[0].to_complex()
        for a, val in zip(arrs, t[1:]):
            a[k] = np.uint64(val & 0xFFFFFFFFFFFFFFFF)
    return (v, *arrs)
