"""Index maps of the four-step pass B and its scatter, restated on the CPU.

Pass B accumulates row pair rp (rows rp and N1-rp; rp = 0: rows 0 and N1/2)
into slots a (psrdada_cpp_gb300/csrc/gspec_fourstep_common.cuh: pair_slot);
fourstep_scatter_kernel (gspec_fourstep.cu) maps every output bin c back to
its (rp, a).  Together they must cover the N/2 + 1 bins of the R2C spectrum
exactly once, and the scatter must be the inverse of the slot map.
"""
import pytest


def slot_bin(rp, a, n1, n2):
    """Bin k1 + N1*k2 that slot a of row pair rp holds (pair_slot)."""
    if rp != 0:
        if a < n2 // 2:
            k1, k2 = rp, a
        else:
            k1, k2 = n1 - rp, a - n2 // 2
    elif a <= n2 // 2:
        k1, k2 = 0, a
    else:
        k1, k2 = n1 // 2, a - n2 // 2 - 1
    return k1 + n1 * k2


def scatter_source(c, n1, n2):
    """(rp, a) the scatter kernel reads for output bin c."""
    k1, k2 = c % n1, c // n1
    if k1 == 0:
        return 0, k2
    if k1 == n1 // 2:
        return 0, n2 // 2 + 1 + k2
    if k1 < n1 // 2:
        return k1, k2
    return n1 - k1, n2 // 2 + k2


@pytest.mark.parametrize("n1,n2", [(64, 128), (128, 128), (256, 256), (512, 512), (1024, 1024), (1024, 128)])
def test_slots_cover_every_bin_once_and_scatter_inverts_them(n1, n2):
    n = n1 * n2
    bins = {}
    for rp in range(n1 // 2):
        for a in range(n2 + 1 if rp == 0 else n2):
            c = slot_bin(rp, a, n1, n2)
            assert 0 <= c <= n // 2, (rp, a, c)
            assert c not in bins, f"bin {c} from {(rp, a)} and {bins.get(c)}"
            bins[c] = (rp, a)
    assert len(bins) == n // 2 + 1
    for c, src in bins.items():
        assert scatter_source(c, n1, n2) == src
