"""Packed-index maps (src/indices_norm.F90, src/ord_utils.F90): bit-exact."""
import itertools

import numpy as np

from conftest import load_golden
from oracle import bruteforce as bf
from oracle import oracle as orc


def test_nwords_and_tables():
    for n in range(1, 17):
        assert orc.nwords(n) == n * (n + 1) * (n + 2) * (n + 3) // 24
    lindi, lindj, lindk, normind = orc.index_tables(6)
    for i in range(1, 7):
        assert lindi[i - 1] == (i - 1) * i * (i + 1) * (i + 2) // 24
        assert lindj[i - 1] == (i - 1) * i * (i + 1) // 6
        assert lindk[i - 1] == (i - 1) * i // 2
    for q in itertools.product(range(1, 7), repeat=4):
        assert normind[tuple(x - 1 for x in q)] == bf.normind(*q)


def test_normind_is_a_bijection_on_sorted_quadruples():
    n = 7
    vals = sorted(bf.lindice(*q) for q in itertools.product(range(1, n + 1), repeat=4)
                  if list(q) == sorted(q, reverse=True))
    assert vals == list(range(1, orc.nwords(n) + 1))


def _ord8_python(t):
    """Independent restatement of src/ord_utils.F90:71-129 used as a check."""
    a, b = list(t[:4]), list(t[4:])
    if bf.normind(*a) < bf.normind(*b):
        a, b = b, a
    for i in range(4):
        jmax = max(range(i, 4), key=lambda j: (a[j], -j))
        if jmax != i:
            a[i], a[jmax] = a[jmax], a[i]
            b[i], b[jmax] = b[jmax], b[i]
    return a + b


def test_ord8_ord9_golden():
    g = load_golden("index_maps")
    t = g["tuples"].astype(np.int64)
    np.testing.assert_array_equal(orc.ord_tuples(4, 8, t), g["ord8"].astype(np.int64))
    np.testing.assert_array_equal(orc.ord_tuples(4, 9, t), g["ord9"].astype(np.int64))
    for row, want in zip(t[:500], g["ord8"][:500]):
        assert _ord8_python(row) == list(want)
    np.testing.assert_array_equal(orc.index_tables(5)[3], g["normind5"])


def test_ord8_and_ord9_differ_only_in_partner_order_on_ties():
    g = load_golden("index_maps")
    o8, o9 = g["ord8"].astype(int), g["ord9"].astype(int)
    np.testing.assert_array_equal(o8[:, :4], o9[:, :4])
    differ = np.any(o8[:, 4:] != o9[:, 4:], axis=1)
    keys = o8[:, :4]
    has_tie = np.array([len(set(k)) < 4 for k in keys])
    assert not np.any(differ & ~has_tie)
