"""CPU model of the four-stage tile schedule of the mixed stage groups
(ceda_demonstrations_gb300/csrc/stage_fused.cu), checked against stages applied one at a time.

The model restates the kernel's index logic: a 128 x (TH+8) load window starting at
(x0-4, y0-4) with zero fill outside the grid, stage l of a group of ks computed on the tile
rows [-(ks-1-l), TH+ks-1-l) and on all 128 columns (columns 0 and 127 taking a stand-in for
their missing outer neighbour), each stage written over the d_{j-2} array in place, points
outside the grid zeroed after every stage, and only the 120 x TH output block of the last two
stages stored. The arithmetic is the mixed stage's difference form in FP64 on both sides (the
bit-level FP32 arithmetic is what the GPU tests compare against the oracle); this test pins
the cone, halo, in-place and masking logic on its own."""
import numpy as np
import pytest

FW, FH = 128, 4
FOW = FW - 2 * FH


def stage_point(c, dc, dw, de, ds, dn, m2, q0, fy, fx):
    gs, gx, gy, gm, gF = c
    lx = (dw - dc) + (de - dc)
    ly = (ds - dc) + (dn - dc)
    inc = gs * dc + gx * lx + gy * ly + gm * (dc - m2) + gF * q0 + fy * fx
    return dc + inc


def one_stage_at_a_time(d1, d2, f0, coefs, sx, sy, ks):
    ny, nx = d1.shape
    for c in coefs[:ks]:
        p = np.zeros((ny + 2, nx + 2))
        p[1:-1, 1:-1] = d1
        new = stage_point(c, d1, p[1:-1, :-2], p[1:-1, 2:], p[:-2, 1:-1], p[2:, 1:-1], d2, f0,
                          sy[:, None], sx[None, :])
        d2, d1 = d1, new
    return d2, d1


def tile_schedule(d1, d2, f0, coefs, sx, sy, ks, th, stand_in):
    ny, nx = d1.shape
    ah = th + 2 * FH
    o1 = np.full((ny, nx), np.nan)
    o2 = np.full((ny, nx), np.nan)

    def load(g, x0, y0):
        a = np.zeros((ah, FW))
        ys, xs = y0 - FH, x0 - FH
        r0, r1 = max(0, -ys), min(ah, ny - ys)
        c0, c1 = max(0, -xs), min(FW, nx - xs)
        if r0 < r1 and c0 < c1:
            a[r0:r1, c0:c1] = g[ys + r0:ys + r1, xs + c0:xs + c1]
        return a

    tiles_x = (nx + FOW - 1) // FOW
    for t in range(tiles_x * ((ny + th - 1) // th)):
        x0, y0 = (t % tiles_x) * FOW, (t // tiles_x) * th
        arr0, arr1, f0s = load(d1, x0, y0), load(d2, x0, y0), load(f0, x0, y0)
        gx = np.arange(FW) + x0 - FH
        gy = np.arange(ah) + y0 - FH
        colin = (gx >= 0) & (gx < nx)
        rowin = (gy >= 0) & (gy < ny)
        fx = np.where(colin, sx[np.clip(gx, 0, nx - 1)], 0.0)
        fy = np.where(rowin, sy[np.clip(gy, 0, ny - 1)], 0.0)
        for l in range(ks):
            X, Y = (arr1, arr0) if l & 1 else (arr0, arr1)
            h = ks - 1 - l
            rs = slice(FH - h, FH + th + h)  # array rows of this stage
            cur = X[rs]
            up = X[FH - h - 1:FH + th + h - 1]
            dn = X[FH - h + 1:FH + th + h + 1]
            west = np.empty_like(cur)
            east = np.empty_like(cur)
            west[:, 1:] = cur[:, :-1]
            east[:, :-1] = cur[:, 1:]
            west[:, 0] = stand_in
            east[:, -1] = stand_in
            new = stage_point(coefs[l], cur, west, east, up, dn, Y[rs], f0s[rs], fy[rs][:, None], fx[None, :])
            new = np.where(rowin[rs][:, None] & colin[None, :], new, 0.0)
            Y[rs] = new
            if l >= ks - 2:
                tgt = o1 if l == ks - 1 else o2
                blk = new[h:h + th, FH:FH + FOW]
                yy, xx = min(th, ny - y0), min(FOW, nx - x0)
                tgt[y0:y0 + yy, x0:x0 + xx] = blk[:yy, :xx]
    return o2, o1


@pytest.mark.parametrize("nx,ny", [(8, 8), (132, 33), (248, 70), (364, 130)])
@pytest.mark.parametrize("ks", [2, 3, 4])
@pytest.mark.parametrize("th", [32, 58, 64])
def test_tile_schedule_equals_one_stage_at_a_time(nx, ny, ks, th):
    rng = np.random.default_rng(nx * 1000 + ny * 10 + ks + th)
    d1, d2, f0 = (rng.standard_normal((ny, nx)) for _ in range(3))
    sx, sy = rng.standard_normal(nx), rng.standard_normal(ny)
    coefs = [tuple(rng.uniform(-0.3, 0.3, 5)) for _ in range(ks)]
    r2, r1 = one_stage_at_a_time(d1, d2, f0, coefs, sx, sy, ks)
    # any value may stand in for the columns the tile does not load: a huge one shows that it
    # never reaches the stored block
    e2, e1 = tile_schedule(d1, d2, f0, coefs, sx, sy, ks, th, stand_in=1e300)
    assert np.array_equal(r1, e1) and np.array_equal(r2, e2)


def test_difference_as_sum_of_negation_is_exact():
    """The paired form takes a - b as a + (-b) (mixed_pair in kernels.cuh): IEEE addition of the
    exact negation gives the same FP32 result, signed zeros included."""
    rng = np.random.default_rng(7)
    a = rng.standard_normal(200000).astype(np.float32) * np.float32(10.0) ** rng.integers(-30, 30, 200000).astype(np.float32)
    b = np.where(rng.random(200000) < 0.1, a, rng.standard_normal(200000).astype(np.float32))
    specials = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf], dtype=np.float32)
    a = np.concatenate([a, np.repeat(specials, specials.size)])
    b = np.concatenate([b, np.tile(specials, specials.size)])
    with np.errstate(invalid="ignore", over="ignore"):
        d1 = a - b
        d2 = a + (b * np.float32(-1.0))
    same = (d1.view(np.uint32) == d2.view(np.uint32)) | (np.isnan(d1) & np.isnan(d2))
    assert same.all()
