"""The run kernel's rebuild requests, restated phase by phase on the host.

Between grid barriers a body of the persistent kernel (oxg_kernels.cuh, k_run) does:
read the request (body 0: st.rebuild, left by the run start or the previous launch;
body b > 0: rb[b & 1]); rebuild the lists if set; forces; block 0 clears the request it
read (after the force barrier, when every block has read it); the step phase of body b
sets rb[(b + 1) & 1] (the run start sets st.rebuild) where a particle moved half the
buffer; after the last body block 0 hands rb[bodies & 1] to st.rebuild and clears both.
The invariant checked: every step rebuilds exactly when the step before it flagged a
displacement, across launches of any length, and no request is lost or read twice."""

import numpy as np
import pytest


class _Status:
    def __init__(self):
        self.rebuild = 0
        self.rb = [0, 0]


def _launch(st, bodies, flags, prologue=False, rebuild0=False, moved=False):
    """One launch; flags[b] = some particle moved half the buffer in body b's step
    phase. Returns the per-body rebuild decisions (the run start's first)."""
    done = []
    start = -1 if prologue else 0
    for body in range(start, bodies):
        pro = body < 0
        if pro:
            rebuild = rebuild0 or moved
        else:
            rebuild = (st.rebuild if body == 0 else st.rb[body & 1]) != 0
        done.append(rebuild)
        # ... lists, forces, force barrier ...
        if body == 0:
            st.rebuild = 0
        elif body > 0:
            st.rb[body & 1] = 0
        # step phase
        if flags[body - start]:
            if pro:
                st.rebuild |= 1
            else:
                st.rb[(body + 1) & 1] |= 1
        # step barrier
        if body == bodies - 1:
            st.rebuild = st.rb[bodies & 1]
            st.rb = [0, 0]
    return done


@pytest.mark.parametrize("seed", range(20))
def test_every_step_rebuilds_exactly_after_a_flagged_step(seed):
    rng = np.random.default_rng(seed)
    st = _Status()
    total = int(rng.integers(1, 60))
    flags = rng.random(total + 1) < 0.3  # the run start's step one, then every body
    decisions = []
    # the first launch of the run starts with the run start body
    done, pos = 0, 0
    first = True
    while done < total:
        n = int(rng.integers(1, 9))
        n = min(n, total - done)
        k = n + (1 if first else 0)
        decisions += _launch(st, n, flags[pos:pos + k], prologue=first, rebuild0=first)
        pos += k
        done += n
        first = False
    assert len(decisions) == total + 1
    assert decisions[0]  # new lists at the run start
    # body t rebuilds iff the step before it (t - 1; the run start for t = 1) flagged
    for t in range(1, total + 1):
        assert decisions[t] == bool(flags[t - 1]), (seed, t)
    # what is left after the run is the last step's request, handed to the next run
    assert st.rebuild == int(flags[total]) and st.rb == [0, 0]


def test_a_request_survives_a_launch_boundary():
    st = _Status()
    d1 = _launch(st, 2, [False, False, True], prologue=True, rebuild0=False)
    assert d1 == [False, False, False] and st.rebuild == 1
    d2 = _launch(st, 3, [False, False, False])
    assert d2 == [True, False, False] and st.rebuild == 0
