"""The shared-memory layouts the line kernels rely on, checked exhaustively on
the CPU: the XOR swizzles (csrc/line_impl.cuh swz, csrc/cluster_impl.cuh cswz)
permute each row, put every step of both walks on 32 distinct banks, and give
the register addressing the passes use (node k of a wordline segment at its
first node XOR k, of a bitline segment at Rb[k % V] + k * row length); and the
red-black comparator's thread-to-node map.  The formulas are restated here; a
change in the kernels must be mirrored."""
import pytest

# (LD, NSEG, SEG, LPW, T, V) of line_impl.cuh's LineCfg
LINE = [(128, 4, 32, 8, 512, 8), (64, 4, 16, 8, 256, 8), (32, 4, 8, 8, 128, 8)]


def swz(LD, r, c):
    if LD == 128:
        x = (r & 7) | ((((c >> 5) ^ (r >> 5)) & 3) << 3)
    elif LD == 64:
        x = (r & 7) | ((((c >> 5) & 1) ^ ((r >> 4) & 1)) << 3) | (((r >> 5) & 1) << 4)
    else:
        x = r & 31
    return r * LD + (c ^ x)


@pytest.mark.parametrize("LD,NSEG,SEG,LPW,T,V", LINE)
def test_line_layout(LD, NSEG, SEG, LPW, T, V):
    for r in range(LD):
        assert sorted(swz(LD, r, c) - r * LD for c in range(LD)) == list(range(LD))
    for warp in range(T // 32):
        for k in range(SEG):
            row_walk, col_walk = set(), set()
            for lane in range(32):
                s, line = lane // LPW, warp * LPW + lane % LPW
                row_walk.add(swz(LD, line, s * SEG + k) % 32)
                col_walk.add(swz(LD, s * SEG + k, line) % 32)
            assert len(row_walk) == 32 and len(col_walk) == 32, (warp, k)
    for line in range(LD):
        for s in range(NSEG):
            p0 = s * SEG
            Bw = swz(LD, line, p0)
            Rb = [swz(LD, p0 + t, line) - t * LD for t in range(V)]
            for k in range(SEG):
                assert Bw ^ k == swz(LD, line, p0 + k)
                assert Rb[k % V] + k * LD == swz(LD, p0 + k, line)


def test_input_padding_spreads_the_bitline_walk():
    """vpad: the bitline pass reads rows 16 s + k of NSEG segments at once."""
    vpad = lambda p: p + (p >> 4)
    for LD, NSEG, SEG, _, _, _ in LINE:
        for k in range(SEG):
            assert len({vpad(s * SEG + k) % 32 for s in range(NSEG)}) == NSEG


# (LDM, C, RPC, NSEG_W, LPW_W, NSEG_B, LPW_B, V) of cluster_impl.cuh's CCfg; 512 threads, 32-node segments
CLUSTER = [(256, 4, 64, 8, 4, 2, 16, 4), (512, 16, 32, 16, 2, 1, 32, 2)]


def cswz(LDM, lr, c):
    if LDM == 256:
        x = (lr & 3) | (((c >> 5) & 3) << 2) | ((((c >> 7) ^ (lr >> 5)) & 1) << 4)
    else:
        x = (lr & 1) | (((c >> 5) & 15) << 1)
    return lr * LDM + (c ^ x)


@pytest.mark.parametrize("LDM,C,RPC,NSEG_W,LPW_W,NSEG_B,LPW_B,V", CLUSTER)
def test_cluster_layout(LDM, C, RPC, NSEG_W, LPW_W, NSEG_B, LPW_B, V):
    SEG, T = 32, 512
    for lr in range(RPC):
        assert sorted(cswz(LDM, lr, c) - lr * LDM for c in range(LDM)) == list(range(LDM))
    for warp in range(T // 32):
        for k in range(SEG):
            word = {cswz(LDM, warp * LPW_W + lane % LPW_W, (lane // LPW_W) * SEG + k) % 32 for lane in range(32)}
            bit = {cswz(LDM, (lane // LPW_B) * SEG + k, warp * LPW_B + lane % LPW_B) % 32 for lane in range(32)}
            assert len(word) == 32 and len(bit) == 32, (warp, k)
    for lr in range(RPC):
        for s in range(NSEG_W):
            Bw = cswz(LDM, lr, s * SEG)
            assert all(Bw ^ k == cswz(LDM, lr, s * SEG + k) for k in range(SEG))
    for col in range(LDM):
        for s in range(NSEG_B):
            p0 = s * SEG
            Rb = [cswz(LDM, p0 + t, col) - t * LDM for t in range(V)]
            assert all(Rb[k % V] + k * LDM == cswz(LDM, p0 + k, col) for k in range(SEG))


def test_red_black_sweep_covers_each_colour_once():
    """csrc/rbsor.cu: thread t owns column t % 128 at rows t / 128 + 8k and, in
    half-sweep c, relaxes its cells' wordline node when (row0 + col) & 1 == c,
    else their bitline node.  For every shape up to 128 x 128 each half-sweep
    updates every node of colour c exactly once (wordline (i+j)&1, bitline
    (i+j+1)&1), and every value it reads -- the line neighbours and the
    partner in the other plane -- has the other colour, so the update is a true
    red-black Gauss-Seidel step."""
    import numpy as np
    T, MAXL, STEP = 1024, 128, 8
    t = np.arange(T)
    col, row0 = t % MAXL, t // MAXL
    for n in (2, 3, 5, 8, 9, 16, 31, 64, 77, 100, 127, 128):
        for m in (2, 3, 5, 8, 9, 16, 31, 64, 77, 100, 127, 128):
            for c in (0, 1):
                hitU = np.zeros((n, m), int)
                hitD = np.zeros((n, m), int)
                for tt in range(T):
                    j = col[tt]
                    if j >= m:
                        continue
                    isU = ((row0[tt] + j) & 1) == c
                    rows = np.arange(row0[tt], n, STEP)
                    (hitU if isU else hitD)[rows, j] += 1
                    # reads: line neighbours in the same plane, the partner in the other
                    for i in rows:
                        own = (i + j) & 1 if isU else (i + j + 1) & 1
                        assert own == c
                        nbrs = [(i, j - 1), (i, j + 1)] if isU else [(i - 1, j), (i + 1, j)]
                        for a, b in nbrs:
                            if 0 <= a < n and 0 <= b < m:
                                assert (((a + b) & 1) if isU else ((a + b + 1) & 1)) != c
                        assert (((i + j + 1) & 1) if isU else ((i + j) & 1)) != c
                ii, jj = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
                assert np.array_equal(hitU, (((ii + jj) & 1) == c).astype(int)), (n, m, c)
                assert np.array_equal(hitD, (((ii + jj + 1) & 1) == c).astype(int)), (n, m, c)


def test_cluster_red_black_bands_cover_each_colour_once():
    """csrc/rbsor_cluster.cu: CTA r of a C-CTA cluster holds global rows
    r*RPC ... r*RPC + nloc - 1; its thread t owns column t % LDM at local rows
    t / LDM + (1024 / LDM) k and, in half-sweep c, relaxes its cells' wordline
    node when (r*RPC + t / LDM + col) & 1 == c, else their bitline node.  Over
    all CTAs each half-sweep updates every node of colour c exactly once, and
    every value it reads -- including the halo rows of the neighbouring bands
    -- has the other colour; the halo a band reads is the neighbour's last
    (above) or first (below) local row, inside that band."""
    import numpy as np
    T = 1024
    for LDM, C, RPC in ((256, 4, 64), (512, 16, 32)):
        STEP = T // LDM
        t = np.arange(T)
        col, lr0 = t % LDM, t // LDM
        for n, m in ((LDM, LDM), (130, 256), (200, 150), (LDM - 3, LDM - 1), (300, 420), (129, 7)):
            if max(n, m) > LDM or max(n, m) <= LDM // 2 and LDM == 512:
                continue
            for c in (0, 1):
                hitU = np.zeros((n, m), int)
                hitD = np.zeros((n, m), int)
                for r in range(C):
                    row0 = r * RPC
                    nloc = max(0, min(RPC, n - row0))
                    for tt in range(T):
                        j = col[tt]
                        if j >= m:
                            continue
                        isU = ((row0 + lr0[tt] + j) & 1) == c
                        for lr in range(lr0[tt], nloc, STEP):
                            i = row0 + lr
                            (hitU if isU else hitD)[i, j] += 1
                            own = (i + j) & 1 if isU else (i + j + 1) & 1
                            assert own == c
                            if isU:
                                nbrs = [(i, j - 1), (i, j + 1)]
                            else:
                                nbrs = [(i - 1, j), (i + 1, j)]
                                if lr == 0 and i > 0:  # halo above: the band above is full
                                    assert r > 0 and i - 1 == (r - 1) * RPC + RPC - 1
                                if lr + 1 == nloc and i + 1 < n:  # halo below: the next band's first row
                                    assert r + 1 < C and i + 1 == (r + 1) * RPC
                            for a, b in nbrs:
                                if 0 <= a < n and 0 <= b < m:
                                    assert (((a + b) & 1) if isU else ((a + b + 1) & 1)) != c
                            assert (((i + j + 1) & 1) if isU else ((i + j) & 1)) != c
                ii, jj = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
                assert np.array_equal(hitU, (((ii + jj) & 1) == c).astype(int)), (LDM, n, m, c)
                assert np.array_equal(hitD, (((ii + jj + 1) & 1) == c).astype(int)), (LDM, n, m, c)
