"""The kernels' run ("segment") bookkeeping, restated from cz_codec.cu,
against the reference survivor order (FullWaveletTransform.h:58-96) and the
positional mask index (:86), over every slot of a block."""


def pos_of_stream(s):
    """Reference order: coarse 4^3 in z,y,x, then per level 8,16,32 the
    octant codes 1..7 in z,y,x order (positional coordinates)."""
    if s < 64:
        return s & 3, (s >> 2) & 3, s >> 4
    for lh, base in ((2, 64), (3, 512), (4, 4096)):
        hh = 1 << lh
        if s < base + 7 * hh ** 3:
            r = s - base
            code = r // hh ** 3 + 1
            w = r % hh ** 3
            return (hh * (code & 1) + w % hh, hh * ((code >> 1) & 1) + (w // hh) % hh,
                    hh * ((code >> 2) & 1) + w // (hh * hh))
    raise ValueError(s)


def phys_of_pos(px, py, pz):
    m = max(px, py, pz)
    if m >= 16:
        return py, pz, px
    if m >= 8:
        return pz, px, py
    return px, py, pz


def slot_of(s):
    """cz_codec.cu slot_of: (x,y,z), run index (global), bit."""
    if s < 64:
        return (s & 3, (s >> 2) & 3, s >> 4), 0, 0
    if s < 512:
        q = s - 64
        seg, e = q >> 2, q & 3
        c = (seg >> 4) + 1
        return (4 * (c & 1) + e, 4 * ((c >> 1) & 1) + (seg & 3), 4 * (c >> 2) + ((seg >> 2) & 3)), 1 + seg, e
    if s < 4096:
        q = s - 512
        seg, e = q >> 3, q & 7
        c = (seg >> 6) + 1
        return (8 * (c >> 2) + ((seg >> 3) & 7), 8 * (c & 1) + e, 8 * ((c >> 1) & 1) + (seg & 7)), 113 + seg, e
    q = s - 4096
    seg, e = q >> 4, q & 15
    c = (seg >> 8) + 1
    return (16 * ((c >> 1) & 1) + (seg & 15), 16 * (c >> 2) + ((seg >> 4) & 15), 16 * (c & 1) + e), 561 + seg, e


def emit_runs():
    """Which (run, bit) each physical coefficient lands in, from the emit32/
    emit16/emit8 epilogues; also which mask bit it sets."""
    where, maskbit = {}, {}
    for y in range(32):  # level-32 z lines (x,y)
        for x in range(32):
            chi = 1 | ((x >= 16) << 1) | ((y >= 16) << 2)
            sub = ((y & 15) << 4) | (x & 15)
            for z in range(32):
                if z >= 16:
                    where[(x, y, z)] = (561 + (chi - 1) * 256 + sub, z - 16)
                elif chi > 1:
                    where[(x, y, z)] = (561 + (chi - 2) * 256 + sub, z)
                if z >= 16 or chi > 1:
                    maskbit[(x, y, z)] = 32 * (x + 32 * y) + z
    for z in range(16):  # level-16 y lines (x,z)
        for x in range(16):
            chi = 1 | ((z >= 8) << 1) | ((x >= 8) << 2)
            sub = ((x & 7) << 3) | (z & 7)
            for y in range(16):
                if y >= 8:
                    where[(x, y, z)] = (113 + (chi - 1) * 64 + sub, y - 8)
                elif chi > 1:
                    where[(x, y, z)] = (113 + (chi - 2) * 64 + sub, y)
                if y >= 8 or chi > 1:
                    maskbit[(x, y, z)] = 32 * (z + 32 * x) + y
    for z in range(8):  # level-8 x lines (y,z)
        for y in range(8):
            chi = 1 | ((y >= 4) << 1) | ((z >= 4) << 2)
            sub = ((z & 3) << 2) | (y & 3)
            for x in range(8):
                if x >= 4:
                    where[(x, y, z)] = (1 + (chi - 1) * 16 + sub, x - 4)
                elif chi > 1:
                    where[(x, y, z)] = (1 + (chi - 2) * 16 + sub, x)
                maskbit[(x, y, z)] = 32 * (y + 32 * z) + x
    return where, maskbit


def test_slots_follow_reference_order_and_runs():
    where, maskbit = emit_runs()
    seen_pos, seen_bits = set(), set()
    last = (-1, -1)
    for s in range(32768):
        px, py, pz = pos_of_stream(s)
        phys = phys_of_pos(px, py, pz)
        got, run, e = slot_of(s)
        assert got == phys
        seen_pos.add(phys)
        # mask bit = positional index
        assert maskbit[phys] == px + 32 * (py + 32 * pz)
        seen_bits.add(maskbit[phys])
        if s >= 64:
            assert where[phys] == (run, e)
            # runs appear in increasing order along the stream, bits in order
            assert (run, e) > last
            last = (run, e)
    assert len(seen_pos) == 32768 and len(seen_bits) == 32768
