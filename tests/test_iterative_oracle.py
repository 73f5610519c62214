"""The oracle's DOS.readjust rules (seqCS.ml:680-722) and select_one
(sequence.ml:1143-1156) on hand-worked cases."""
import numpy as np

from oracle import oracle as O


def test_select_one_takes_the_lowest_state():
    m = O.cm_dna(1, 2, -1)
    s = np.array([16, 3, 12, 15, 17, 8], np.uint8)
    assert O.select_one(s, m).tolist() == [16, 1, 4, 1, 1, 8]


def test_empty_neighbour_rules():
    m = O.cm_dna(1, 2, -1)
    e = np.array([16], np.uint8)
    a = np.array([16, 1, 2, 4], np.uint8)
    b = np.array([16, 1, 4], np.uint8)
    mine = np.array([16, 2], np.uint8)
    for mode in ("three", "approx"):
        assert O.dos_readjust(mode, e, e, a, mine, m)[1].tolist() == [16]      # ch1
        assert O.dos_readjust(mode, e, b, e, mine, m)[1].tolist() == [16]      # ch1
        assert O.dos_readjust(mode, a, e, e, mine, m)[1].tolist() == [16]      # ch2
        # one empty: the selected median of the other two, align_2's cost
        ch, res, cost = O.dos_readjust(mode, a, b, e, mine, m)
        c2, ra, rb = O.align_2(a, b, m)
        assert cost == c2 and res.tolist() == O.select_one(O.median_2(ra, rb, m), m).tolist()
        assert ch
    # unchanged median: changed is False
    ch, res, _ = O.dos_readjust("three", a, a, a, a, m)
    assert not ch and res.tolist() == a.tolist()


def test_host_select_one_matches_oracle():
    # the GPU module's select_one (host numpy) against the oracle's
    from poyd_gb300 import iterative
    m = O.cm_dna(1, 2, -1)
    rng = np.random.default_rng(2)
    s = rng.integers(1, 32, size=200).astype(np.uint8)
    s[0] = 16
    assert np.array_equal(iterative.select_one(s, None), O.select_one(s, m))
