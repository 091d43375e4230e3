"""Basis persistence (save / load_basis): definitions round-trip on CPU; representatives and
the matvec after loading on the GPU."""

import numpy as np
import pytest

from ls_helpers import LAT, ls


def bases():
    return [
        ls.SpinBasis(16, 8, -1, ls.Symmetries(LAT.chain_symmetries(16, 3, None))),
        ls.SpinBasis(12, 6, None, ls.Symmetries(LAT.chain_symmetries(12, 0, 1))),
        ls.SpinBasis(10),
        ls.SpinfulFermionBasis(8, (4, 3)),
        ls.SpinfulFermionBasis(9, (3, 3), symmetries=ls.Symmetries(LAT.square_symmetries(3, 0, 0, True))),
        ls.SpinlessFermionBasis(10, 4),
    ]


def test_definitions_round_trip():
    for b in bases():
        obj = b.json_object()
        c = ls.basis_from_json(obj)
        assert c.json_object() == obj
        assert type(c) is type(b)
        assert c.number_bits == b.number_bits
        assert c._estimates() == b._estimates()


@pytest.mark.gpu
def test_save_load_matvec(tmp_path):
    import torch
    for i, b in enumerate(bases()[:5]):
        b.build()
        path = str(tmp_path / "basis{}.npz".format(i))
        b.save(path)
        c = ls.load_basis(path)
        assert np.array_equal(np.asarray(c.states), np.asarray(b.states))
        expr = LAT.xxz(LAT.chain_bonds(b.number_spins), 1.0, 0.5) if isinstance(b, ls.SpinBasis) else \
            LAT.hubbard(LAT.square_bonds(3) if b.number_sites == 9 else LAT.chain_bonds(b.number_sites), 1.0, 4.0,
                        number_sites=b.number_sites)
        D = b.number_states
        x = torch.from_numpy(np.random.default_rng(i).normal(size=D) + 0.5j).cuda()
        y1 = ls.Operator(b, expr).apply_device(x)
        y2 = ls.Operator(c, expr).apply_device(x)
        assert torch.equal(y1, y2)
        assert np.array_equal(c.index(np.asarray(b.states)), np.arange(D))
