"""GCF choice per w-region (host logic of librc_gb300, no GPU) against the
oracle's restatement of gcfGet / gcfKernel."""
import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import gcf as G
from rc_gb300 import lib


def test_select_matches_reference_rule():
    rng = np.random.default_rng(0)
    files = [0.0, 50.0, 100.0, 100.0, 400.0, 250.0]
    for _ in range(300):
        w0, w1 = sorted(rng.uniform(-600, 600, 2))
        assert G.select(files, w0, w1) == O.gcf_select(files, w0, w1)
    # ties: the last of equal maxima; conjugation for mostly-negative regions
    assert G.select(files, 120.0, 130.0) == (3, False)
    assert G.select(files, -300.0, 10.0) == (5, True)


def test_select_without_candidate_is_an_error():
    with pytest.raises(lib.GbError):
        G.select([10.0, 20.0], 1.0, 5.0)
