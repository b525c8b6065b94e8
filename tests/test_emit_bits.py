"""The packed level extraction of bs_emit_dist (msbfs.cu emit_vertex4_packed)
restated on the CPU: for every source, the level assembled from eight-source
bytes of the level slices with one multiply must equal the level read bit by
bit, and unreached pairs must come out as -1.  Integer arithmetic, so the
check is exact."""

import numpy as np

M32 = 0xFFFFFFFF


def packed_levels(vis, slices, nsrc):
    """Levels of one vertex's word as the kernel computes them (uint32 math)."""
    nb = len(slices)
    out = []
    for c in range(8):
        if 8 * c >= nsrc:
            break
        packed = 0
        for k in range(min(nb, 4)):
            packed |= ((slices[k] >> (8 * c)) & 0xFF) << (8 * k)
        five = (slices[4] >> (8 * c)) & 0xFF if nb > 4 else 0
        vb = (vis >> (8 * c)) & 0xFF
        for b in range(min(8, nsrc - 8 * c)):
            x = ((((packed >> b) & 0x01010101) * 0x01020408) & M32) >> 24
            if nb > 4:
                x |= ((five >> b) & 1) << 4
            v = (x | ((((vb >> b) & 1) - 1) & M32)) & M32
            out.append(v - (1 << 32) if v >= 1 << 31 else v)
    return out


def bitwise_levels(vis, slices, nsrc):
    out = []
    for s in range(nsrc):
        if not (vis >> s) & 1:
            out.append(-1)
            continue
        out.append(sum(((w >> s) & 1) << k for k, w in enumerate(slices)))
    return out


def test_packed_matches_bitwise():
    rng = np.random.default_rng(5)
    for nb in range(1, 6):
        for trial in range(300):
            vis = int(rng.integers(0, 1 << 63)) | (int(rng.integers(0, 2)) << 63)
            sl = [int(rng.integers(0, 1 << 63)) | (int(rng.integers(0, 2)) << 63) for _ in range(nb)]
            for nsrc in (64, 63, 9, 8, 1):
                assert packed_levels(vis, sl, nsrc) == bitwise_levels(vis, sl, nsrc), (nb, trial, nsrc)
    # extremes: every bit set, none set
    full = (1 << 64) - 1
    for nb in range(1, 6):
        assert packed_levels(full, [full] * nb, 64) == [(1 << nb) - 1] * 64
        assert packed_levels(0, [full] * nb, 64) == [-1] * 64
        assert packed_levels(full, [0] * nb, 64) == [0] * 64
