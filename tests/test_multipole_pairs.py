"""Host logic of the degree pairs: which m = 0 terms one paired fields pass
and contraction serve."""
from pyhermes_gb300 import multipole as mp


def _lms(l_min, l_max):
    return [(l, m) for l in range(l_min, l_max + 1) for m in range(l + 1)]


def test_pairs_even_degree_with_the_next():
    assert mp.degree_pairs(_lms(0, 10)) == [0, 2, 4, 6, 8]
    assert mp.degree_pairs(_lms(0, 6)) == [0, 2, 4]
    assert mp.degree_pairs(_lms(0, 0)) == []


def test_pairs_need_both_degrees():
    # l_min = 1: degree 1 has no even partner below it, 10 none above
    assert mp.degree_pairs(_lms(1, 10)) == [2, 4, 6, 8]
    assert mp.degree_pairs(_lms(3, 3)) == []
    assert mp.degree_pairs([(0, 0), (2, 0), (3, 1)]) == []
    assert mp.degree_pairs([(4, 0), (5, 0)]) == [4]
