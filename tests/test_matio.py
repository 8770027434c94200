"""Faust .mat files: the MAT5 'faust_factors' cell of Transform::save_mat_file /
read_from_mat_file (src/faust_linear_operator/CPU/faust_Transform.hpp:434-514),
tested like the reference's save/load round trips (pyfaust test_FaustPy.py
testSave: save, load, same product)."""
import numpy as np
import pytest
import scipy.io as sio
import scipy.sparse as sp

from faust_gb300 import _ffi, matio
from faust_gb300.faust import BSRFactor


class _HostFaust:
    """Host stand-in with the accessors matio.save reads (no device needed)."""

    def __init__(self, factors=None, bsr=None):
        self._f = factors or []
        self._b = bsr or []
        self.dtype_code = _ffi.BF16 if bsr else (_ffi.F32 if factors[0].dtype == np.float32 else _ffi.F64)

    def numfactors(self):
        return len(self._b or self._f)

    def factors(self, i):
        return sp.csr_matrix(self._f[i])

    def bsr_factor(self, i):
        return self._b[i]


def _rand_csr(rng, m, n, dt, density=0.2):
    return sp.random(m, n, density=density, format="csr", dtype=dt, random_state=rng)


def _rand_bsr(rng, rows, cols, per_row):
    nbr, nbc = rows // 64, cols // 64
    bcol = np.concatenate([np.sort(rng.choice(nbc, per_row, replace=False)) for _ in range(nbr)]).astype(np.int32)
    brow = np.arange(0, nbr * per_row + 1, per_row, dtype=np.int32)
    vals = rng.standard_normal((bcol.size, 64, 64)).astype(np.float32)
    bits = (vals.view(np.uint32) >> 16).astype(np.uint16)  # truncation: exact bf16 values
    return BSRFactor(rows, cols, brow, bcol, bits)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_save_layout_csr(tmp_path, dt):
    """1 x J cell of MATLAB sparse matrices, single for float32 and double for
    float64 (MatSparse::toMatIOVar), factor order kept."""
    rng = np.random.default_rng(1)
    facs = [_rand_csr(rng, 30, 20, dt), _rand_csr(rng, 20, 20, dt), _rand_csr(rng, 20, 45, dt)]
    p = str(tmp_path / "f.mat")
    matio.save(_HostFaust(facs), p)
    assert [w[0] for w in sio.whosmat(p)] == ["faust_factors"]
    cell = sio.loadmat(p)["faust_factors"]
    assert cell.shape == (1, 3)
    for got, want in zip(cell[0], facs):
        assert sp.issparse(got) and got.dtype == dt and got.shape == want.shape
        assert (abs(sp.csr_matrix(got) - want)).max() == 0


def test_save_layout_bsr(tmp_path):
    """A BSR factor is the 1 x 5 cell {'bsr', [rows cols nblocks], bcolinds,
    browptr, 64 x nblocks*64 column-major blocks} of MatBSR::toMatIOVar."""
    rng = np.random.default_rng(2)
    b = _rand_bsr(rng, 256, 192, 2)
    p = str(tmp_path / "b.mat")
    matio.save(_HostFaust(bsr=[b]), p)
    c = sio.loadmat(p)["faust_factors"][0, 0]
    assert c.shape == (1, 5) and str(c[0, 0][0]) == "bsr"
    assert c[0, 1].dtype == np.int32 and list(c[0, 1].ravel()) == [256, 192, b.nnz_blocks]
    assert np.array_equal(c[0, 2].ravel(), b.bcolind) and np.array_equal(c[0, 3].ravel(), b.browptr)
    data = c[0, 4]
    assert data.dtype == np.float32 and data.shape == (64, 64 * b.nnz_blocks)
    # block j, entry (r, c) at data[r, j*64 + c]
    j, r, col = 3, 5, 17
    want = (np.array([b.blocks_colmajor[j, col, r]], np.uint32) << 16).view(np.float32)[0]
    assert data[r, j * 64 + col] == want
    back = matio._load_bsr(c)
    assert np.array_equal(back.blocks_colmajor, b.blocks_colmajor)
    assert np.array_equal(back.browptr, b.browptr) and np.array_equal(back.bcolind, b.bcolind)


def test_bf16_rounding_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, np.inf, np.nan], np.float32)
    bits = matio._f32_to_bf16(x)
    assert list(bits[:5]) == [0x3F80, 0x3F80, 0x3F82, 0xC020, 0x7F80]
    assert bits[5] == 0x7FC0


def test_load_rejects_non_cell(tmp_path):
    p = str(tmp_path / "x.mat")
    sio.savemat(p, {"faust_factors": np.ones((2, 2))})
    with pytest.raises(ValueError):
        matio.load(p)
    sio.savemat(p, {"other": np.ones((2, 2))})
    with pytest.raises(ValueError):
        matio.load(p)


@pytest.mark.gpu
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_roundtrip_csr_gpu(tmp_path, dt):
    """save -> load gives the same factors and a bit-identical product."""
    from faust_gb300 import Faust
    rng = np.random.default_rng(3)
    facs = [_rand_csr(rng, 64, 48, dt), _rand_csr(rng, 48, 48, dt), _rand_csr(rng, 48, 80, dt)]
    F = Faust(facs, dtype=dt)
    p = str(tmp_path / "f.mat")
    F.save(p)
    G = Faust.load(p)
    assert G.shape == F.shape and G.numfactors() == 3 and G.dtype == np.dtype(dt)
    for i in range(3):
        assert (abs(G.factors(i) - F.factors(i))).max() == 0
    X = rng.standard_normal((80, 7)).astype(dt)
    assert np.array_equal(F @ X, G @ X)
    F.close()
    G.close()


@pytest.mark.gpu
def test_roundtrip_dense_cell_gpu(tmp_path):
    """A dense cell (MatDense::toMatIOVar) loads as a factor with its zeros dropped."""
    from faust_gb300 import Faust
    rng = np.random.default_rng(4)
    A = rng.standard_normal((16, 16))
    A[A < 0.3] = 0
    B = _rand_csr(rng, 16, 24, np.float64)
    cell = np.empty((1, 2), dtype=object)
    cell[0, 0], cell[0, 1] = A, B.tocsc()
    p = str(tmp_path / "d.mat")
    sio.savemat(p, {"faust_factors": cell})
    G = Faust.load(p)
    assert G.factors(0).nnz == np.count_nonzero(A)
    assert np.array_equal(G.factors(0).toarray(), A)
    G.close()


@pytest.mark.gpu
def test_roundtrip_bsr_gpu(tmp_path):
    from faust_gb300 import Faust
    rng = np.random.default_rng(5)
    F = Faust([_rand_bsr(rng, 256, 256, 2), _rand_bsr(rng, 256, 128, 1)])
    p = str(tmp_path / "b.mat")
    F.save(p)
    G = Faust.load(p)
    assert G.shape == F.shape and G.numfactors() == 2
    for i in range(2):
        a, b = F.bsr_factor(i), G.bsr_factor(i)
        assert np.array_equal(a.blocks_colmajor, b.blocks_colmajor) and np.array_equal(a.bcolind, b.bcolind)
    F.close()
    G.close()
