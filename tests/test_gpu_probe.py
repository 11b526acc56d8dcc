"""The cache read-bandwidth probe behind the bench's roofline (dl_probe_read_bandwidth): on the
GPU it reports a positive L2 read rate for a buffer that fits in L2, and an L1 rate (each block
re-reading its own 32 KiB slice) at least as high."""
import ctypes as C

import pytest

import dynlight_gb300 as dl

pytestmark = pytest.mark.gpu


def test_probe_reads_l2_and_l1():
    lib = dl.load_library()
    l2, l1 = C.c_double(), C.c_double()
    assert lib.dl_probe_read_bandwidth(0, 2, 64 << 20, 20, C.byref(l2)) == 0, lib.dl_last_error()
    assert lib.dl_probe_read_bandwidth(0, 1, 64 << 20, 80, C.byref(l1)) == 0, lib.dl_last_error()
    # a GB300's L2 streams several TB/s; far from any plausible rate means the probe is broken
    assert 1000.0 < l2.value < 200000.0, l2.value
    assert l1.value >= 0.9 * l2.value, (l1.value, l2.value)
