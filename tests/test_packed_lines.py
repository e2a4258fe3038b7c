"""Order lines packed in 4 bytes for the host link (ltpg_tpcc_pack_lines,
host code): i_id in bits 0..16, supply_w in 17..27, qty in 28..31; round trip
on generated batches, and a line out of range is refused (no GPU needed)."""
import numpy as np
import pytest

from ltpg_gb300 import LtpgError, TpccBatch, TpccGenerator


@pytest.mark.parametrize("w", [1, 64, 2047])
def test_pack_round_trip(w):
    g = TpccGenerator(5, w, 3000)
    b = g.next()
    p = b.with_packed_lines()
    assert p.n_lines == b.n_lines and p.nbytes() == b.n_txn * 32 + b.n_lines * 4
    q = p.packed
    assert np.array_equal(q & 0x1FFFF, b.lines["i_id"])
    assert np.array_equal((q >> 17) & 0x7FF, b.lines["supply_w"])
    assert np.array_equal(q >> 28, b.lines["qty"])


@pytest.mark.parametrize("field,value", [("i_id", 1 << 17), ("supply_w", 1 << 11), ("qty", 16)])
def test_pack_refuses_a_line_out_of_range(field, value):
    b = TpccGenerator(6, 4, 500).next()
    bad = TpccBatch(b.txns, b.lines.copy(), b.txn_base)
    bad.lines[field][min(3, bad.n_lines - 1)] = value
    with pytest.raises(LtpgError):
        bad.with_packed_lines()
    bad.lines[field][min(3, bad.n_lines - 1)] = value - 1  # the largest that fits
    bad.with_packed_lines()
