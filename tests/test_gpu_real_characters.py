"""The real-element shortcut of the matvec kernels: characters whose imaginary parts are at most
1e-14 count as real (cos/sin(-2 pi phi) leave residues of ~1e-16 in sectors such as (pi, pi)),
and a complex right-hand side then takes 2 FP64 FMAs per element instead of 4.  Here the
characters of a real sector are perturbed on both sides of that threshold; the GPU result must
match the oracle's complex scatter with the same perturbed characters to 1e-12 either way (below
the threshold the dropped parts are below 1e-14 of every element)."""

import numpy as np
import pytest

import oracle as O
from ls_helpers import LAT, Case, ls

pytestmark = pytest.mark.gpu


class _Perturbed(ls.Symmetries):
    """A symmetry group whose characters carry an extra imaginary part `delta` on every element
    except the identity."""

    delta = 0.0

    @property
    def characters(self):
        re, im = super().characters
        im = im.copy()
        ident = np.all(self.permutations == np.arange(self.number_bits), axis=1)
        im[~ident] += self.delta * np.where(np.arange(len(im))[~ident] % 2 == 0, 1.0, -1.0)
        return re, im


@pytest.mark.parametrize("delta", [0.0, 5e-15, 2e-14, 1e-12])
def test_characters_across_the_real_threshold(delta):
    import torch
    syms = _Perturbed(LAT.chain_symmetries(16, 8, 1))
    syms.delta = delta
    basis = ls.SpinBasis(16, 8, -1, syms)
    case = Case(basis, LAT.heisenberg(LAT.chain_bonds(16)), "chain16")
    re, im = syms.characters
    # the oracle group with the same (perturbed) characters, in the product's element order
    case.group = O.Group(syms.permutations, re, im, -1, 16, *syms.network())
    basis.build()
    states = basis.states
    x = np.random.default_rng(3).normal(size=len(states)) + 1j * np.random.default_rng(4).normal(size=len(states))
    y = case.op.apply_device(torch.from_numpy(x).cuda()).cpu().numpy()
    yo = case.oracle_matvec(states, x, complex_=True)
    assert np.linalg.norm(y - yo) / np.linalg.norm(yo) <= 1e-12
