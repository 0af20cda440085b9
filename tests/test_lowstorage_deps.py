"""The low-storage kernel's neighbour-flag synchronisation (rk_gb300/csrc/rkcu_lowstorage.cu):
the CTA ranges a CTA waits for before a wavefront step must include every CTA whose slice
holds a pair its stencils read, and every CTA whose stencils read its slice (so that a ring
slot is not overwritten while a neighbour still reads it).  The ranges below restate the
kernel's formulas; the check enumerates every slice's reads by brute force."""
import itertools


def wait_ranges(c, G, N, R):
    """The kernel's ranges: CTA c holds block positions [c R N / G, (c+1) R N / G) of every
    block (truncated in a shorter last block)."""
    nb = (N + R - 1) // R
    npf = R * N
    owner = lambda q: ((q + 1) * G - 1) // npf
    out = []
    a, e = c * npf // G, (c + 1) * npf // G
    if a < e:
        k0, k1 = a // N, (e - 1) // N
        out.append((owner((k0 - 1) * N if k0 > 0 else 0), owner((k1 + 2) * N - 1 if k1 + 2 < R else npf - 1)))
        if k0 == 0 and nb > 1:
            out.append((owner((R - 1) * N), G - 1))
        if k1 == R - 1 and nb > 1:
            out.append((0, owner(N - 1)))
    return out


def reads(c, G, N, R):
    """CTAs holding the pairs that c's stencils read: rows k +- 1 in the same column and the
    same row's columns j +- 1, across block edges."""
    nb = (N + R - 1) // R
    npf = R * N
    owner = lambda loc: ((loc + 1) * G - 1) // npf
    out = set()
    for b in range(nb):
        np_b = min(R, N - b * R) * N
        for q in range(min(np_b, c * npf // G), min(np_b, (c + 1) * npf // G)):
            k, j = divmod(q, N)
            gk = b * R + k
            for dk, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                gk2, j2 = gk + dk, j + dj
                if 0 <= gk2 < N and 0 <= j2 < N:
                    out.add(owner((gk2 % R) * N + j2))
    out.discard(c)
    return out


def test_wait_ranges_cover_reads_and_readers():
    for N, R, G in itertools.product((2, 3, 8, 33, 100), (1, 3, 16, 64), (1, 7, 37, 100)):
        if R > 2 * N:
            continue
        need = {c: reads(c, G, N, R) for c in range(G)}
        for c in range(G):
            cover = set()
            for lo, hi in wait_ranges(c, G, N, R):
                cover |= set(range(lo, hi + 1))
            readers = {x for x in range(G) if c in need[x]}
            assert need[c] <= cover, (N, R, G, c, sorted(need[c] - cover))
            assert readers <= cover, (N, R, G, c, sorted(readers - cover))
