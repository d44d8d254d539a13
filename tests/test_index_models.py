"""Index models of two kernels whose addressing is not a plain grid walk,
checked on the CPU for many grid shapes (ragged ones included), as they were
before the kernels first ran:

* k_advect_tma (csrc/k_advect.cu): every shared-memory read of the staged
  phi tile (40 x 14 x 14 floats per block: x from the 16-byte-aligned column
  before the tile's first halo column, 14 rows j0-3..j0+10, 14 levels
  k0-3..k0+10) stays inside the tile, for lanes inside and outside the grid;
* k_sor_odd_seg (csrc/k_sweep.cu): segments decode to valid (row, column
  tile, level range), every segment a block waits for exists, holds an
  earlier ticket and publishes its value, and the launch fits the context's
  chain arrays (odd_chain_segments);
* k_sor_odd_seg<double>'s marching production phase reads the same x
  points and records as the level-per-warp form it replaced.

The models restate the kernels' index arithmetic line by line."""
import pytest

XOFF = 3
AT_BX, AT_BY, AT_TZ, AT_W, AT_NR, AT_NZ = 32, 8, 8, 40, 14, 14
SOC_SC = 64


def _tma_reads(nx, ny, nz):
    """Yields (column, row, level) of every staged read of k_advect_tma."""
    for bx in range((nx + AT_BX - 1) // AT_BX):
        for by in range((ny + AT_BY - 1) // AT_BY):
            for bz in range((nz + AT_TZ - 1) // AT_TZ):
                i0, j0, k0 = bx * AT_BX + 1, by * AT_BY + 1, bz * AT_TZ + 1
                k1, x0 = min(k0 + AT_TZ - 1, nz), bx * AT_BX
                for ty in range(AT_BY):
                    for tx in range(AT_BX):
                        ii, jj, rown = i0 + tx, j0 + ty, ty + 3

                        def ph(c, r, kk):
                            return (c + XOFF - x0, r, kk - k0 + 3)

                        def xf(iu, r, kp):
                            if 3 <= iu <= nx - 2:
                                return [ph(iu + d, r, kp) for d in range(-2, 4)]
                            return [ph(iu, r, kp), ph(iu + 1, r, kp)]

                        def yf(ip, jv, kp):
                            rb = jv - j0 + 1
                            return [ph(ip, rb + d, kp) for d in range(6)]

                        for d in range(-3, 3):
                            yield ph(ii, rown, k0 + d)
                        for k in range(k0, k1 + 1):
                            yield ph(ii, rown, k + 3)
                            yield from xf(ii, rown, k)
                            yield from yf(ii, jj, k)
                            if ty == 0:
                                yield from yf(ii, j0 - 1, k)
                            elif ty == 1 and tx < AT_BY:
                                yield from xf(i0 - 1, tx + 3, k)


@pytest.mark.parametrize("size", [(64, 32, 48), (37, 5, 23), (70, 19, 9), (33, 17, 31), (8, 6, 12),
                                  (130, 9, 17)])
def test_tma_staged_reads_stay_in_the_tile(size):
    bad = [r for r in _tma_reads(*size) if not (0 <= r[0] < AT_W and 0 <= r[1] < AT_NR and 0 <= r[2] < AT_NZ)]
    assert not bad, bad[:5]


def _odd_chain_segments(nx, ny, nz):
    gx = (((nx + 1) // 2) + 31) // 32
    return ((nz - 1) // SOC_SC + 1) * gx * ny


@pytest.mark.parametrize("size", [(256, 128, 192), (512, 256, 256), (64, 32, 200), (37, 19, 150), (8, 6, 400),
                                  (33, 17, 31), (4, 3, 4), (384, 192, 192), (192, 96, 144), (5, 3, 129)])
def test_segment_chain_waits_on_earlier_publishing_segments(size):
    nx, ny, nz = size
    cap = _odd_chain_segments(nx, ny, nz)
    for comp in (0, 1, 2):
        iend = nx - 1 if comp == 0 else nx
        gx = ((iend + 1) // 2 + 31) // 32
        k0, k1 = (1 if comp == 2 else 0), nz - 1
        nseg = (nz - 1 - k0) // SOC_SC + 1
        grid, nct = nseg * gx * ny, gx * ny
        assert grid <= cap
        published = set()
        for t in range(grid):  # tickets in the order blocks take them
            seg, ct = divmod(t, nct)
            bx, j = ct % gx, ct // gx + 1
            assert 0 <= bx < gx and 1 <= j <= ny
            kc = k0 + seg * SOC_SC
            n = min(SOC_SC, k1 - kc + 1)
            assert 1 <= n and kc + n - 1 <= k1
            if seg > 0:
                assert t - nct in published  # an earlier ticket, already publishing
            if seg < (k1 - k0) // SOC_SC:
                published.add(t)
        assert max(published, default=-1) < cap


def _odd_reads(nx, ny, nz, comp, march):
    """Global reads of one odd half-sweep's production phase over every
    segment of every column tile: the x points (column, row, level) and the
    record slots (level of a record read), for the level-per-warp form
    (march False) or the FP64 marching form; also checks the shared-memory
    rows each form writes stay inside the 64-level segment."""
    SOC_W = 8
    PER = SOC_SC // SOC_W
    iend = nx - 1 if comp == 0 else nx
    npair = (iend + 1) // 2
    k0, k1 = (1 if comp == 2 else 0), nz - 1
    xs, recs = set(), set()
    for j in range(1, ny + 1):
        par = (j + 1) & 1  # flg = 1; the other parity only shifts i
        for i2 in range(npair):
            i = 2 * i2 + 1 + par
            if i > iend:
                continue
            for kc in range(k0, k1 + 1, SOC_SC):
                n = min(SOC_SC, k1 - kc + 1)
                for w in range(SOC_W):
                    if march:
                        lb, le = w * PER, min(n, w * PER + PER)
                        levels = list(range(lb, le))
                        if levels:
                            xs.add((i, j, kc + lb))  # the first centre value
                    else:
                        levels = [w + r * SOC_W for r in range(PER) if w + r * SOC_W < n]
                    for lk in levels:
                        assert 0 <= lk < SOC_SC
                        k = kc + lk
                        recs.add((i, j, k))
                        if not march:
                            xs.add((i, j, k))
                        if comp == 2 or k != nz - 1:
                            xs.add((i, j, k + 1))
                        xs.update({(i + 1, j, k), (i - 1, j, k), (i, j + 1, k), (i, j - 1, k)})
                        if k == k0 and comp == 2:
                            xs.add((i, j, k - 1))
    return xs, recs


@pytest.mark.parametrize("size", [(16, 6, 192), (13, 5, 150), (8, 3, 64), (9, 4, 200), (6, 3, 65)])
@pytest.mark.parametrize("comp", [0, 1, 2])
def test_fp64_marching_odd_sweep_reads_what_the_level_form_reads(size, comp):
    """k_sor_odd_seg<double>'s marching production (each warp walks its own
    8 levels, the point above a level reused as the next centre value)
    reads exactly the x points and records of the level-per-warp form, so
    it reads nothing the earlier form did not."""
    nx, ny, nz = size
    xs_l, recs_l = _odd_reads(nx, ny, nz, comp, False)
    xs_m, recs_m = _odd_reads(nx, ny, nz, comp, True)
    assert recs_m == recs_l
    assert xs_m == xs_l
    assert all(0 <= p[2] <= nz for p in xs_m)
