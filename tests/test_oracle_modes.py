"""The oracle's two modes, both pinned to the reference CPU backend.

The GPU stream is compared with the oracle run with reference quirks off
(`oracle_set_reference_quirks(0)`).  That mode differs from the reference
build in exactly two places, both where the reference delivers stale buffer
contents:

1. the tail of a partial final epoch: the reference leaves whatever the
   previous user of the buffer wrote there (the pool slot of the same batch
   position, src/cpu/stream.c:623-629; for a pyramid the linear epoch
   buffer of the previous epoch), quirks-off writes the fill value 0;
2. the dim-0 drain at flush when epochs-per-batch K equals a level's period
   2^l: the reference delivers the slot its planned shard-order table names
   (src/cpu/pipeline.c:14-31, 152-172), which holds the previous period's
   emission, quirks-off delivers the drained accumulation.

These tests show that quirks-off equals the reference everywhere else:
on every stream shape of the parity suite, and on inputs that make the
stale bytes equal the corrected ones (a zero previous occupant of the
buffer; epochs repeating so that a partial period reduces like a full one),
with the differences on general inputs confined to the predicted shards.
"""
import numpy as np
import pytest

import cases
import harness as H
from chucky_gb300 import capi

needs_ref = pytest.mark.skipif(H.reference() is None,
                               reason="reference build (oracle/_ref) not present")

DTYPES = ["u16", "i8", "f32", "u64"]


def _stale_free(cfg, data, epochs):
    """Zero the epochs whose buffers the partial final epoch inherits: every
    earlier epoch at the same batch position, and the epoch just before it
    (the pyramid's linear buffer)."""
    if float(epochs).is_integer():
        return data
    info = H.plan_info(cfg)
    K = int(info.epochs_per_batch)
    ee = int(info.epoch_elements)
    last = int(epochs)
    out = data.copy()
    for e in range(last):
        if e % K == last % K or e == last - 1:
            out[e * ee:(e + 1) * ee] = 0
    return out


@needs_ref
@pytest.mark.parametrize("case", cases.CASES, ids=[c[0] for c in cases.CASES])
@pytest.mark.parametrize("dtype", DTYPES)
def test_quirks_off_equals_reference(case, dtype):
    cfg, epochs = cases.build(case, dtype)
    n = int(epochs * H.epoch_elements(cfg))
    data = _stale_free(cfg, cases.make_data(dtype, n, seed=7), epochs)
    ref, cr = H.run_reference(cfg, data)
    on, con = H.run_oracle(cfg, data, quirks=True)
    off, coff = H.run_oracle(cfg, data, quirks=False)
    assert cr == con == coff
    assert on == ref, H.diff_shards(on, ref)
    assert off == ref, H.diff_shards(off, ref)


@needs_ref
@pytest.mark.parametrize("dtype", DTYPES)
def test_partial_tail_is_the_only_divergence(dtype):
    """On general input the two modes differ only in shards that hold the
    partial final epoch (found by changing that epoch's values in the
    reference run)."""
    case = cases.CASES[[c[0] for c in cases.CASES].index("partial_epoch")]
    cfg, epochs = cases.build(case, dtype)
    ee = H.epoch_elements(cfg)
    n = int(epochs * ee)
    data = cases.make_data(dtype, n, seed=7)
    ref, _ = H.run_reference(cfg, data)
    off, _ = H.run_oracle(cfg, data, quirks=False)
    assert off != ref  # the stale tail is visible on this input
    bumped = data.copy()
    last = int(epochs) * ee
    bumped[last:] = cases.make_data(dtype, n - last, seed=99)
    ref2, _ = H.run_reference(cfg, bumped)
    holds_last = {k for k in ref if ref[k] != ref2.get(k)}
    differing = {k for k in set(ref) | set(off) if ref.get(k) != off.get(k)}
    assert differing and differing <= holds_last, (differing, holds_last)


def _drain_case(K):
    """u16 frames with a 3-level (t, y, x) max pyramid folded along dim 0,
    K epochs per batch: level log2(K) has period K."""
    D = dict
    dims = capi.make_dims([D(size=0, chunk=4, cps=1, downsample=1),
                           D(size=36, chunk=8, cps=2, downsample=1),
                           D(size=64, chunk=8, cps=4, downsample=1)])
    cfg = capi.make_config(dims, dtype="u16", reduce="max", append_reduce="max",
                           max_nlod=3, epochs_per_batch=K)
    cfg._dims = dims
    return cfg


@needs_ref
@pytest.mark.parametrize("K,epochs", [(2, 5), (2, 7), (4, 6), (4, 9)])
def test_drain_at_level_period_pinned_on_repeating_epochs(K, epochs):
    """Every epoch holds the same values, so with max the drained partial
    period reduces to the previous period's emission: all three agree even
    though the drain of level log2(K) triggers."""
    cfg = _drain_case(K)
    ee = H.epoch_elements(cfg)
    one = cases.make_data("u16", ee, seed=3)
    data = np.tile(one, epochs)
    ref, _ = H.run_reference(cfg, data)
    on, _ = H.run_oracle(cfg, data, quirks=True)
    off, _ = H.run_oracle(cfg, data, quirks=False)
    assert on == ref, H.diff_shards(on, ref)
    assert off == ref, H.diff_shards(off, ref)


@needs_ref
@pytest.mark.parametrize("K,epochs", [(2, 5), (4, 6)])
def test_drain_divergence_confined_to_the_drained_level(K, epochs):
    cfg = _drain_case(K)
    ee = H.epoch_elements(cfg)
    data = cases.make_data("u16", epochs * ee, seed=5)
    ref, _ = H.run_reference(cfg, data)
    off, _ = H.run_oracle(cfg, data, quirks=False)
    on, _ = H.run_oracle(cfg, data, quirks=True)
    assert on == ref, H.diff_shards(on, ref)
    level = K.bit_length() - 1  # period 2^level == K
    differing = {k for k in set(ref) | set(off) if ref.get(k) != off.get(k)}
    assert differing, "the drain should differ on random input"
    assert {k[0] for k in differing} == {level}, differing
