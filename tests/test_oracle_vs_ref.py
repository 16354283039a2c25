"""Live comparison of the oracle restatement with the reference build
(oracle/_ref, only where the reference sources were present at build time)."""
import math

import numpy as np
import pytest

PHI = 0.25 * math.pi


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.reference_available():
        pytest.skip("reference build (oracle/_ref) not present")
    return oracle


@pytest.mark.parametrize("L,channel,q,neel,steps", [
    (6, 0, (0, 0), 0.1, 3000), (8, 0, (0, 0), 0.0, 3000), (10, 0, (0, 0), 0.05, 2000),
    (4, 1, (2, 2), 0.1, 2000), (8, 1, (2, 2), 0.1, 800),
    # long exciton: states two orbital hops apart in one flavour (rank-2 row updates)
    (4, 2, (0, 0), 0.1, 1500), (4, 2, (2, 0), 0.1, 1500), (4, 2, (1, 1), 0.1, 1500), (6, 2, (2, 2), 0.1, 600)])
def test_walk_bit_exact(ref, L, channel, q, neel, steps):
    o = ref.OracleChain(L, PHI, neel, channel=channel, q=q, seed=42, walker=1)
    r = ref.RefChain(L, PHI, neel, channel=channel, q=q, seed=42, walker=1)
    assert o.random_start() == r.random_start() == 0
    to, tr = o.walk(steps, trace=True), r.walk(steps, trace=True)
    for f in ("v1", "v2", "kind", "accepted"):
        assert (to[f] == tr[f]).all()
    assert (to["ratio"] == tr["ratio"]).all()
    np.testing.assert_array_equal(o.config(), r.config())
    assert o.amp() == r.amp()
    o.walk(L * L * 4, meas=L * L, mask=1)
    r.walk(L * L * 4, meas=L * L, mask=1)
    np.testing.assert_array_equal(o.projheis()[0], r.projheis()[0])
