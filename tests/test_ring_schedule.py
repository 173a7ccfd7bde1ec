"""The schedule of the mixed path's accumulator rings, restated on the host
with the kernels' index arithmetic (k_coefecheby / k_flux_deriv slot =
iteration mod S; k_flux_flush: slice p = (k mod S) / q flushed over all S slots
when k mod q = q - 1, and at a read every slice's pending window
(now - s) mod S < (now - p q - q + 1) mod S, then the C slots cleared; the Cvj
ring is the case P = 1, q = S = 32).  Random runs with reads, gated iterations
(C slot 0) and iteration jumps (a read first): every (point, iteration) is
added exactly once."""
import random

import pytest


def simulate(NF, S, P, ops):
    q = S // P
    chunk = (NF + P - 1) // P
    cring = [None] * S                  # id of the iteration whose C_k is in the slot (None: zero)
    fring = [[None] * NF for _ in range(S)]
    added = [dict() for _ in range(NF)]
    expected = [set() for _ in range(NF)]
    uid = 0
    it = 0

    def add(f, k):
        added[f][k] = added[f].get(k, 0) + 1

    def final(now):
        for f in range(NF):
            p = f // chunk
            npend = (now - (p * q + q - 1)) % S
            for s in range(S):
                if (now - s) % S < npend and cring[s] is not None:
                    assert fring[s][f] == cring[s]
                    add(f, cring[s])
        for s in range(S):
            cring[s] = None

    for op in ops:
        if op[0] == "iter":
            it += 1
            uid += 1
            s = it % S
            gated = op[1]
            cring[s] = None if gated else uid
            if not gated:
                for f in range(NF):
                    fring[s][f] = uid
                    expected[f].add(uid)
            if it % q == q - 1:
                p = (it % S) // q
                for f in range(p * chunk, min(NF, (p + 1) * chunk)):
                    for s2 in range(S):
                        if cring[s2] is not None:
                            assert fring[s2][f] == cring[s2]
                            add(f, cring[s2])
        elif op[0] == "read":
            final(it)
        else:                           # upload of a state at another iteration
            final(it)
            it = op[1]
    final(it)
    for f in range(NF):
        assert set(added[f]) == expected[f]
        assert all(v == 1 for v in added[f].values())


@pytest.mark.parametrize("seed", range(4))
def test_every_sample_is_added_once(seed):
    rng = random.Random(seed)
    for _ in range(100):
        S = rng.choice([8, 16, 32])
        P = rng.choice([p for p in (1, 2, 4, 8, 16, 32) if p <= S])
        ops = []
        for _ in range(rng.randint(1, 150)):
            r = rng.random()
            if r < 0.86:
                ops.append(("iter", rng.random() < 0.1))
            elif r < 0.96:
                ops.append(("read",))
            else:
                ops.append(("jump", rng.randint(0, 90)))
        simulate(rng.randint(1, 40), S, P, ops)
