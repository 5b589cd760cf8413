"""The copy schedule of the shared-memory staging of the symmetric products
(SliceStager in csrc/krylov.cu), replayed on the CPU.

Each warp streams the column and value planes of its slices w0, w0 + nw, ...
(empty slices skipped) into a ring of NST stages of at most CH slots.  The
producer issues chunk c into stage c % NST and the consumer waits for phase
c // NST of that stage's barrier.  This replay follows the same cursor
arithmetic and checks, for random slice widths (zeros included) and launch
shapes: the consumer reads exactly the chunks the producer wrote, in order;
a stage is refilled only after it was consumed; every copy is 16-byte
aligned, a multiple of 16 bytes, inside the arrays, and below the mbarrier
transaction limit; and no copy is left in flight at the end.
"""
import numpy as np
import pytest

SLOT_COL_BYTES = 32 * 4        # 32 int32 columns per slot
SLOT_VAL_BYTES = 32 * 9 * 4    # 32 x 9 float values per slot
TX_LIMIT = (1 << 20) - 1       # mbarrier transaction count


def replay(sptr, nwarps, CH, NST):
    ns = len(sptr) - 1
    total_slots = int(sptr[-1])
    for w0 in range(nwarps):
        # producer cursor
        st = {"ps": w0, "pk": 0, "pb0": 0, "pw": 0, "pidx": 0}
        stages = [None] * NST          # chunk held by each stage: (slice, first slot, slots, phase)

        def seek():
            while st["ps"] < ns:
                st["pb0"] = int(sptr[st["ps"]])
                st["pw"] = int(sptr[st["ps"] + 1]) - st["pb0"]
                if st["pw"] > 0:
                    break
                st["ps"] += nwarps
            st["pk"] = 0

        def produce():
            if st["ps"] >= ns:
                return
            s_ = st["pidx"] % NST
            # a stage is refilled only after its previous chunk was consumed
            assert stages[s_] is None, "stage overwritten before it was read"
            nsl = min(CH, st["pw"] - st["pk"])
            first = st["pb0"] + st["pk"]
            col_off, val_off = first * SLOT_COL_BYTES, first * SLOT_VAL_BYTES
            col_len, val_len = nsl * SLOT_COL_BYTES, nsl * SLOT_VAL_BYTES
            assert col_off % 16 == 0 and val_off % 16 == 0 and col_len % 16 == 0 and val_len % 16 == 0
            assert 0 < nsl <= CH and first + nsl <= total_slots
            assert col_len + val_len <= TX_LIMIT
            stages[s_] = (st["ps"], st["pk"], nsl, st["pidx"] // NST)
            st["pidx"] += 1
            st["pk"] += nsl
            if st["pk"] >= st["pw"]:
                st["ps"] += nwarps
                seek()

        seek()
        for _ in range(NST):
            produce()
        cidx = 0
        s = w0
        while s < ns:
            b0, w = int(sptr[s]), int(sptr[s + 1]) - int(sptr[s])
            if w > 0:
                for k in range(0, w, CH):
                    s_ = cidx % NST
                    held = stages[s_]
                    assert held is not None, "waiting on a stage nothing was issued to"
                    assert held == (s, k, min(CH, w - k), cidx // NST), (held, s, k)
                    stages[s_] = None
                    produce()
                    cidx += 1
            s += nwarps
        assert cidx == st["pidx"], "copies left in flight"
        assert all(x is None for x in stages)


@pytest.mark.parametrize("CH,NST", [(2, 4), (1, 4), (3, 3), (4, 2), (2, 5)])
def test_schedule_random_widths(CH, NST):
    rng = np.random.default_rng(CH * 10 + NST)
    for trial in range(40):
        ns = int(rng.integers(1, 60))
        widths = rng.integers(0, 20, ns)
        widths[rng.random(ns) < 0.2] = 0          # empty slices
        sptr = np.concatenate([[0], np.cumsum(widths)]).astype(np.int64)
        nwarps = int(rng.integers(1, 80))           # fewer or more warps than slices
        replay(sptr, nwarps, CH, NST)


def test_schedule_fem_like_widths():
    """Upper-half widths of a hex8 pattern (up to 14 blocks per row) over
    3,000 slices and the 2 CTAs x 8 warps x 152 SMs of the solves' launch."""
    rng = np.random.default_rng(7)
    widths = rng.integers(8, 15, 3000)
    sptr = np.concatenate([[0], np.cumsum(widths)]).astype(np.int64)
    replay(sptr, 2 * 8 * 152, 2, 4)
