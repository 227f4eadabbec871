"""CPU checks of index arithmetic the CUDA kernels rely on, restated in
Python from csrc/fl_multigrid.cu:

- the POST smoother's shared prolongation: a region row's two cells (the odd
  column GX + 2tx, GX = bx*T - H with H odd and T even, and the even one after
  it) read coarse columns A = clamp(I, 0, cnx-1) and B = clamp(I+1, 0, cnx-1),
  I = (GX + 2tx - 1) / 2, as (A, B) and (B, A); that must equal each cell's
  own (I, I2) of pressureMultigrid.ts's prolongation for every cell inside
  the grid, and A, B must lie inside the coarse level for every pair;
- the coarse level sizes ceil(n / 2), which that pairing assumes.
"""


def coarse(n):
    return (n + 1) // 2


def own_columns(gi, cnx):
    i = gi >> 1
    i2 = min(i + 1, cnx - 1) if gi & 1 else max(i - 1, 0)
    return i, i2


def test_prolongation_pairs_read_the_same_coarse_columns():
    checked = 0
    for P in (1, 2, 3, 4):
        H = 2 * P + 1
        for R in (32, 64):
            T = R - 2 * H
            assert T % 2 == 0 and T > 0
            for nx in list(range(2, 80)) + [127, 128, 129, 511, 512, 513, 1024]:
                cnx = coarse(nx)
                for bx in range((nx + T - 1) // T):
                    GX = bx * T - H
                    assert GX % 2 == 1 or GX % 2 == -1
                    for tx in range(R // 2):
                        gi0 = GX + 2 * tx
                        I = (gi0 - 1) // 2  # exact: gi0 - 1 is even
                        A = min(max(I, 0), cnx - 1)
                        B = max(min(I + 1, cnx - 1), 0)
                        assert 0 <= A < cnx and 0 <= B < cnx
                        for gi, mine in ((gi0, (A, B)), (gi0 + 1, (B, A))):
                            if 0 <= gi < nx:
                                assert own_columns(gi, cnx) == mine, (P, R, nx, bx, tx, gi)
                                checked += 1
    assert checked > 50000
