"""Input adapters: CSR -> cbtd on the device (gbdpcg_csr_to_cbtd_*), the
layout step behind the reference's CSR overload of solvePCG
(include/interface.cuh:8-20, a stub that exits in the reference)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr_from_cbtd(O, M, n, N, dup=False):
    """Rows of the n N x n N matrix from its cbtd block rows (the padding blocks
    of knots 0 and N-1 are not entries); with dup, every entry is split in two."""
    rp, ci, va = [0], [], []
    for r in range(n * N):
        k, i = divmod(r, n)
        for b in range(3):
            kc = k + b - 1
            if kc < 0 or kc >= N:
                continue
            for j in range(n):
                v = M[k * 3 * n * n + (b * n + j) * n + i]
                if v != 0:
                    if dup:
                        h = M.dtype.type(v * 0.5)
                        ci += [kc * n + j, kc * n + j]
                        va += [h, M.dtype.type(v - h)]
                    else:
                        ci.append(kc * n + j)
                        va.append(v)
        rp.append(len(ci))
    return np.array(rp, np.uint32), np.array(ci, np.uint32), np.array(va, M.dtype)


def _expected(M, n, N):
    """cbtd with the padding blocks zeroed (what the scatter produces)."""
    E = M.copy().reshape(N, 3 * n * n)
    E[0, 0:n * n] = 0
    E[N - 1, 2 * n * n:] = 0
    return E.reshape(-1)


def _dev(a):
    import torch
    t = torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a)
    return t.to(torch.device("cuda:0"))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,N", [(14, 32), (6, 1), (5, 9), (24, 64)])
def test_csr_to_cbtd_matches_layout(gb, oracle_mod, handle, dt, n, N):
    import torch
    O = oracle_mod
    M = O.generate(n, N, 11).cbtd(dt)
    rp, ci, va = _csr_from_cbtd(O, M, n, N)
    out = torch.full((3 * n * n * N,), 7.0, dtype=torch.float64 if dt == np.float64 else torch.float32,
                     device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    gb.csr_to_cbtd(_dev(rp), _dev(ci), _dev(va), n, N, out, err)
    assert out.cpu().numpy().tobytes() == _expected(M, n, N).tobytes()


def test_csr_duplicates_add(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    n, N = 6, 10
    M = O.generate(n, N, 2).cbtd(np.float64)
    rp, ci, va = _csr_from_cbtd(O, M, n, N, dup=True)
    out = torch.empty(3 * n * n * N, dtype=torch.float64, device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    gb.csr_to_cbtd(_dev(rp), _dev(ci), _dev(va), n, N, out, err)
    assert np.array_equal(out.cpu().numpy(), _expected(M, n, N))


def test_csr_entry_outside_band_is_rejected(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    n, N = 4, 6
    M = O.generate(n, N, 1).cbtd(np.float32)
    rp, ci, va = _csr_from_cbtd(O, M, n, N)
    # row 0 (knot 0) gets an entry in knot 3's columns
    rp2 = rp.copy()
    rp2[1:] += 1
    ci2 = np.concatenate([[3 * n + 1], ci]).astype(np.uint32)
    va2 = np.concatenate([[np.float32(1.0)], va]).astype(np.float32)
    out = torch.empty(3 * n * n * N, device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    with pytest.raises(gb.GbdpcgError) as e:
        gb.csr_to_cbtd(_dev(rp2), _dev(ci2), _dev(va2), n, N, out, err)
    assert e.value.code == gb.ERR_INVALID_ARGUMENT
    # the in-band entries are still in place
    exp = _expected(M, n, N)
    assert out.cpu().numpy().tobytes() == exp.tobytes()


@pytest.mark.parametrize("n,N", [(24, 16), (7, 5), (40, 3)])
def test_csr_ragged_and_empty_rows(gb, oracle_mod, handle, n, N):
    """A random half of the band's entries dropped, some rows left empty; n = 40
    takes the one-thread-per-row path (tiles above 32 x 96 do not fit)."""
    import torch
    O = oracle_mod
    M = O.generate(n, N, 5).cbtd(np.float32)
    rng = np.random.default_rng(n * 100 + N)
    keep = rng.random(M.size) < 0.5
    for r in rng.choice(n * N, size=max(1, n * N // 7), replace=False):  # empty rows
        k, i = divmod(int(r), n)
        keep[k * 3 * n * n + i:(k + 1) * 3 * n * n:n] = False
    Md = np.where(keep, M, np.float32(0)).astype(np.float32)
    rp, ci, va = _csr_from_cbtd(O, Md, n, N)
    assert (np.diff(rp.astype(np.int64)) == 0).any()
    out = torch.full((3 * n * n * N,), 7.0, device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    gb.csr_to_cbtd(_dev(rp), _dev(ci), _dev(va), n, N, out, err)
    assert out.cpu().numpy().tobytes() == _expected(Md, n, N).tobytes()


def _dense_from_cbtd(M, n, N, dt):
    D = np.zeros((n * N, n * N), dt)
    for k in range(N):
        for b in range(3):
            kc = k + b - 1
            if 0 <= kc < N:
                blk = M[k * 3 * n * n + b * n * n:k * 3 * n * n + (b + 1) * n * n].reshape(n, n).T  # (i, j)
                D[k * n:(k + 1) * n, kc * n:(kc + 1) * n] = blk
    return D


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("row_major", [False, True])
@pytest.mark.parametrize("n,N,pad", [(14, 9, 0), (5, 4, 3), (24, 3, 8), (32, 2, 0), (6, 1, 0)])
def test_dense_to_cbtd_matches_layout(gb, oracle_mod, handle, dt, row_major, n, N, pad):
    """Dense (column- or row-major, leading dimension n N + pad) -> cbtd, bit
    for bit, padding blocks zero; the band check passes on a banded matrix."""
    import torch
    O = oracle_mod
    M = O.generate(n, N, 13).cbtd(dt)
    D = _dense_from_cbtd(M, n, N, dt)
    ld = n * N + pad
    buf = np.full((n * N, ld), np.nan, dt)  # row-major storage with ld columns
    if row_major:
        buf[:, :n * N] = D
    else:
        buf[:, :n * N] = D.T  # row c of buf = column c of D
    tdt = torch.float64 if dt == np.float64 else torch.float32
    out = torch.full((3 * n * n * N,), 7.0, dtype=tdt, device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    Dd = torch.from_numpy(np.ascontiguousarray(buf)).to("cuda:0")
    if pad:
        # the band check reads only the n N x n N part; NaN padding is not an entry
        gb.dense_to_cbtd(Dd, n, N, out, row_major=row_major, ld=ld)
    else:
        gb.dense_to_cbtd(Dd, n, N, out, row_major=row_major, ld=ld, err=err)
    torch.cuda.synchronize()
    assert out.cpu().numpy().tobytes() == _expected(M, n, N).tobytes()


def test_dense_entry_outside_band_is_rejected(gb, oracle_mod, handle):
    import torch
    O = oracle_mod
    n, N = 4, 5
    M = O.generate(n, N, 3).cbtd(np.float32)
    D = _dense_from_cbtd(M, n, N, np.float32)
    D[1, 3 * n + 2] = 0.5  # knot 0's row, knot 3's column
    out = torch.empty(3 * n * n * N, device="cuda:0")
    err = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    with pytest.raises(gb.GbdpcgError) as e:
        gb.dense_to_cbtd(torch.from_numpy(D).to("cuda:0"), n, N, out, row_major=True, err=err)
    assert e.value.code == gb.ERR_INVALID_ARGUMENT
    # without the check the band is still extracted
    gb.dense_to_cbtd(torch.from_numpy(D).to("cuda:0"), n, N, out, row_major=True)
    torch.cuda.synchronize()
    assert out.cpu().numpy().tobytes() == _expected(M, n, N).tobytes()
