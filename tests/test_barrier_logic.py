"""The run kernel's grid-barrier arithmetic, restated on the host (uint32 wraparound):
block 0 adds 2^31 - (blocks - 1), every other block adds 1, so bit 31 of the counter
flips exactly when the last block arrives, in any arrival order. Between barriers the
counter holds 0 or 2^31 (every completed barrier adds exactly 2^31, the allocation
clears it, and the host clears it again after a launch whose wait gave up), so it needs
no reset between launches. A waiter leaves when bit 31 differs from the value before
its own arrival."""

import itertools

import numpy as np
import pytest

M = 1 << 32
BIT = 1 << 31


def _add(blocks, b):
    return (BIT - (blocks - 1)) % M if b == 0 else 1


@pytest.mark.parametrize("blocks", [2, 3, 4, 5])
def test_phase_flips_exactly_on_the_last_arrival(blocks):
    for start in (0, BIT):  # the counter values between barriers
        for order in itertools.permutations(range(blocks)):
            c = start
            tokens = {}
            for k, b in enumerate(order):
                tokens[b] = c
                c = (c + _add(blocks, b)) % M
                released = [((tokens[x] ^ c) & BIT) != 0 for x in tokens]
                if k < blocks - 1:
                    assert not any(released), (start, order, k)
                else:
                    assert all(released), (start, order)
            # a completed barrier adds exactly 2^31: the next barrier needs no reset
            assert (c - start) % M == BIT


def test_many_consecutive_barriers_and_launches():
    rng = np.random.default_rng(0)
    blocks = 304
    c = 0
    for _ in range(200):  # barriers, across any number of launches
        start = c
        order = rng.permutation(blocks)
        toks = []
        for k, b in enumerate(order):
            toks.append(c)
            c = (c + _add(blocks, int(b))) % M
            if k < blocks - 1:
                assert not any(((t ^ c) & BIT) for t in toks)
        assert all(((t ^ c) & BIT) for t in toks)
        assert (c - start) % M == BIT and c % BIT == 0


def test_missing_block_never_releases():
    """The stalled barrier of the bounded-wait self-test: with one block absent the bit
    never flips, so every waiter runs into its poll limit."""
    for blocks in (2, 3, 8, 304):
        for skip in {0, 1, blocks - 1}:
            c = BIT
            toks = []
            for b in range(blocks):
                if b == skip:
                    continue
                toks.append(c)
                c = (c + _add(blocks, b)) % M
            assert not any(((t ^ c) & BIT) for t in toks)
