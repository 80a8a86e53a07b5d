"""Host buffers: the huge-page check that decides between registered
huge-page memory and cudaHostAlloc (no GPU needed for the parser)."""

from actx_dgfem_suite_gb300.hostmem import huge_page_fraction

SMAPS = """\
7f0000000000-7f0040000000 rw-p 00000000 00:00 0
Size:            1048576 kB
AnonHugePages:    524288 kB
7f0040000000-7f0040200000 rw-p 00000000 00:00 0
Size:               2048 kB
AnonHugePages:         0 kB
555500000000-555500100000 r-xp 00000000 08:01 42   /usr/bin/python3
Size:               1024 kB
AnonHugePages:         0 kB
"""


def test_huge_page_fraction_weights_overlapping_mappings():
    base = 0x7F0000000000
    gib = 1 << 30
    assert abs(huge_page_fraction(base, gib, SMAPS) - 0.5) < 1e-12
    # half of the first mapping plus the second (no huge pages)
    frac = huge_page_fraction(base + gib // 2, gib // 2 + (2 << 20), SMAPS)
    assert abs(frac - (gib // 4) / (gib // 2 + (2 << 20))) < 1e-12
    assert huge_page_fraction(0x555500000000, 1 << 20, SMAPS) == 0.0
    assert huge_page_fraction(0x1000, 4096, SMAPS) == 0.0        # not mapped
    assert huge_page_fraction(base, gib, "") == 0.0
