"""Restricted subspaces on the host: the drop-in classes evaluate a restriction callable
(``restrict_subspace(configuration, replacement)``, tetragono/tetragono/sampling_lattice/sampling.py:133-136)
once per table entry and hand the device one allow flag per entry; restrictions that look at sites
outside the replaced ones cannot be flagged and are refused."""
import numpy as np
import pytest

from tnsp_gb300.lattice import neel, random_heisenberg, table_arrays
from tnsp_gb300.sampling import restriction_flags


def restrict_Sz(configuration, replacement=None):
    """tetraku's total-Sz restriction (tetraku/tetraku/models/heisenberg/restrict_Sz.py:20-58), replacement
    form: the replaced sites keep their number of up spins (EdgePoint index 0)."""
    old = sum(1 for p in replacement if configuration[p][1] == 0)
    new = sum(1 for v in replacement.values() if v[1] == 0)
    return old == new


def test_total_sz_restriction_allows_every_heisenberg_move():
    lat = random_heisenberg(3, 3, 2, seed=1)
    flags = restriction_flags(lat, lat._hamiltonians, restrict_Sz, neel(3, 3))
    assert flags.size == table_arrays(2, lat._hamiltonians)[4].size
    assert flags.all()


def test_flags_follow_the_table_entries():
    """A restriction forbidding every replacement that puts an up spin first disallows exactly the table
    entries whose first output is 0, in table order."""
    lat = random_heisenberg(3, 3, 2, seed=1)
    flags = restriction_flags(lat, lat._hamiltonians, lambda c, r: list(r.values())[0][1] != 0, neel(3, 3))
    outs = table_arrays(2, lat._hamiltonians)[4]
    np.testing.assert_array_equal(flags, (outs // 2 != 0).astype(np.uint8))


def test_edge_points_of_a_charged_physical_edge():
    """U(1) lattices: the physical edge has one index per charge (+1, -1), so every EdgePoint index is 0, as in
    the reference's Bose U(1) points; the total-Sz restriction then allows everything."""
    lat = random_heisenberg(2, 2, None, seed=3, sectors=(1, 1, 1))
    seen = []
    restriction_flags(lat, lat._hamiltonians, lambda c, r: seen.extend(r.values()) or True, neel(2, 2))
    assert set(seen) == {(1, 0), (-1, 0)}


def test_restriction_reading_other_sites_is_refused():
    lat = random_heisenberg(3, 3, 2, seed=1)
    with pytest.raises(NotImplementedError):
        restriction_flags(lat, lat._hamiltonians, lambda c, r: c[2, 2, 0][1] == 0, neel(3, 3))
