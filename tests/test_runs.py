"""The kernels' run ("segment") bookkeeping, restated from cz_block.cuh,
against the reference survivor order (FullWaveletTransform.h:58-96) and the
positional mask index (:86), over every slot of a block; and the warp
iteration that visits the survivors of a block (for_each_survivor)."""
import numpy as np


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


def run_pos(r, e):
    """cz_block.cuh run_pos: physical (x,y,z) of bit e of global run r."""
    if r < 113:
        q = r - 1
        c = (q >> 4) + 1
        return 4 * (c & 1) + e, 4 * ((c >> 1) & 1) + (q & 3), 4 * (c >> 2) + ((q >> 2) & 3)
    if r < 561:
        q = r - 113
        c = (q >> 6) + 1
        return 8 * (c >> 2) + ((q >> 3) & 7), 8 * (c & 1) + e, 8 * ((c >> 1) & 1) + (q & 7)
    q = r - 561
    c = (q >> 8) + 1
    return 16 * ((c >> 1) & 1) + (q & 15), 16 * (c >> 2) + ((q >> 4) & 15), 16 * (c & 1) + e


def slot_of(s):
    """Stream slot s -> (x,y,z), global run index, bit: runs of 4 (level 8),
    8 (level 16) and 16 (level 32) consecutive slots, positions by run_pos."""
    if s < 64:
        return (s & 3, (s >> 2) & 3, s >> 4), 0, 0
    if s < 512:
        run, e = 1 + ((s - 64) >> 2), (s - 64) & 3
    elif s < 4096:
        run, e = 113 + ((s - 512) >> 3), (s - 512) & 7
    else:
        run, e = 561 + ((s - 4096) >> 4), (s - 4096) & 15
    return run_pos(run, e), run, e


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


def run_geom(r):
    """cz_block.cuh run_geom: bit e of run r sits at base + e * stride of the
    padded block layout x + 33 y + 1057 z."""
    x, y, z = run_pos(r, 0)
    stride = 1 if r < 113 else (33 if r < 561 else 1057)
    return x + 33 * y + 1057 * z, stride


def emit_order(masks, off, S):
    """cz_block.cuh emit_survivors: runs 1..2352 in groups of 32 (one per
    lane); each lane copies its run's survivors (ascending bits) to the
    warp's stage at o - first + i, the warp hands stage[b] out as stream
    index first + b. Returns [(k, padded position)]."""
    out = [(t, t % 4 + 33 * ((t >> 2) % 4) + 1057 * (t >> 4)) for t in range(64)]
    for r0 in range(1, 2353, 32):
        rs = [r for r in range(r0, min(r0 + 32, 2353))]
        first = off[rs[0]]
        total = off[rs[-1]] + bin(masks[rs[-1]]).count("1") - first
        stage = [None] * 512
        for r in rs:
            base, stride = run_geom(r)
            i = off[r] - first
            for e in range(16):
                if (masks[r] >> e) & 1:
                    stage[i] = base + e * stride
                    i += 1
        out += [(first + b, stage[b]) for b in range(total)]
    return out


def test_survivor_emission_follows_the_reference_order():
    rng = np.random.default_rng(5)
    widths = [4] * 112 + [8] * 448 + [16] * 1792
    for density in (0.0, 0.05, 0.3, 0.9, 1.0):
        masks = [0]
        for w in widths:
            bits = rng.random(w) < density
            masks.append(int(sum(1 << i for i in range(w) if bits[i])))
        off = [0] * 2353
        acc = 64
        for r in range(1, 2353):
            off[r] = acc
            acc += bin(masks[r]).count("1")
        S = acc
        # the reference order: stream slots in order, the kept ones numbered
        want = []
        for slot in range(32768):
            (x, y, z), run, e = slot_of(slot)
            if slot < 64 or (masks[run] >> e) & 1:
                want.append((len(want), x + 33 * y + 1057 * z))
        assert sorted(emit_order(masks, off, S)) == want
