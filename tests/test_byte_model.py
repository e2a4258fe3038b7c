"""The benchmark's byte model (no GPU): the figures the roofline divides by.
Each late-read setting's kernels account for the same logical bytes where
they do the same work, and only the reads scale with the commit rate."""
import pytest

import bench


@pytest.mark.parametrize("k,u", [(16, 0.05), (10, 0.5), (4, 0.0)])
def test_ycsb_byte_model(k, u):
    early = bench.ycsb_bytes_per_txn(k, u, 0.5)
    assert early[0] == 4 * k + 16 * u * k + 96 * (1 - u) * k + 8  # op words, slots, rows, result
    assert early[2] == early[3] == 0.0
    l1, l2, l3 = (bench.ycsb_bytes_per_txn(k, u, 0.5, late=x) for x in (1, 2, 3))
    # the registration-only execute of late 1 and 2 reads no row
    assert l1[0] == l2[0] == 4 * k + 16 * k
    # late 1 does the reads inside the check kernel: check + reads of late 2
    # (late 2 also reads the flag byte)
    assert l1[1] == pytest.approx(l2[1] + l2[2] - 1)
    # the same reads for late 2 and 3; late 3's write-back also writes the
    # final flag and the bitmap
    assert l3[2] == pytest.approx(l2[2])
    assert l3[3] == pytest.approx(l2[3] + 1 + 1 / 8)
    # rows scale with the commit rate, registration does not
    lo, hi = bench.ycsb_bytes_per_txn(k, u, 0.25, late=3), bench.ycsb_bytes_per_txn(k, u, 0.75, late=3)
    assert lo[0] == hi[0] and lo[1] == hi[1]
    assert hi[2] - lo[2] == pytest.approx(0.5 * (4 * k + 80 * (1 - u) * k))


@pytest.mark.parametrize("n_slots,steps,start", [(32, 20, 5), (32, 400, 20), (8, 8, 0), (8, 3, 7), (1, 5, 0)])
def test_step_chunks_cover_the_steps_in_slot_order(n_slots, steps, start):
    """The timed region's calls: consecutive slots from `start`, wrapping at
    n_slots, no call past the last slot.  The graph warm-up runs each distinct
    call once, so the timed region holds no capture."""
    chunks = bench.step_chunks(n_slots, steps, start)
    slots = [s + j for s, c in chunks for j in range(c)]
    assert slots == [(start + i) % n_slots for i in range(steps)]
    assert all(s + c <= n_slots and c > 0 for s, c in chunks)
    assert len(set(chunks)) <= 3
