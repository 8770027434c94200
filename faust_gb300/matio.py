"""MATLAB .mat (MAT5) storage of a Faust, the file format of
Transform::save_mat_file / read_from_mat_file
(src/faust_linear_operator/CPU/faust_Transform.hpp:434-514).

Layout (kept identical so files move between both libraries):
  * one variable, ``faust_factors``: a 1 x J cell, factor 0 first;
  * a CSR factor is a MATLAB sparse matrix whose values are single for a
    float32 Faust and double for a float64 one (MatSparse::toMatIOVar);
  * a BSR factor is a 1 x 5 cell {'bsr', int32 [rows cols nblocks],
    int32 bcolinds (1 x nblocks), int32 browptr (1 x rows/bh + 1),
    data (bh x nblocks*bw, column-major blocks side by side)}
    (MatBSR::toMatIOVar, faust_MatBSR.hpp:387-470); BF16 values are written
    widened to single, which is exact, and read back rounded to nearest even;
  * a dense cell is read as a factor with its zeros dropped.
The element type of a file is that of its first factor
(Transform::get_mat_file_type, faust_Transform.hpp:517-546).

Host-side file I/O around the device Faust; no arithmetic of the product
runs here.
"""
import numpy as np

VAR = "faust_factors"


def _bf16_to_f32(bits):
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def _f32_to_bf16(x):
    """Round float32 values to BF16 bit patterns, nearest even (NaN kept quiet)."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    nan = np.isnan(np.asarray(x, np.float32))
    r[nan] = 0x7FC0
    return r


def save(F, path):
    """Writes Faust F (all factors) to ``path`` in the layout above."""
    import scipy.io as sio
    from . import _ffi
    n = F.numfactors()
    if n == 0:
        raise ValueError("can't save an empty Faust")
    cell = np.empty((1, n), dtype=object)
    if F.dtype_code == _ffi.BF16:
        for i in range(n):
            cell[0, i] = _bsr_cell(F.bsr_factor(i))
    else:
        for i in range(n):
            cell[0, i] = F.factors(i).tocsc()
    sio.savemat(path, {VAR: cell}, format="5", do_compression=False)


def _bsr_cell(b):
    nb = b.nnz_blocks
    data = _bf16_to_f32(b.blocks_colmajor.reshape(nb * 64, 64)).T  # (64, nb*64): column j*64+c of block j
    c = np.empty((1, 5), dtype=object)
    c[0, 0] = "bsr"
    c[0, 1] = np.array([[b.shape[0], b.shape[1], nb]], np.int32)
    c[0, 2] = b.bcolind.reshape(1, -1).astype(np.int32)
    c[0, 3] = b.browptr.reshape(1, -1).astype(np.int32)
    c[0, 4] = np.asfortranarray(data)
    return c


def _is_bsr_cell(v):
    return (isinstance(v, np.ndarray) and v.dtype == object and v.size == 5
            and np.asarray(v.flat[0]).size and str(np.asarray(v.flat[0]).flat[0]) == "bsr")


def _load_bsr(v):
    from .faust import BSRFactor
    rows, cols, nb = (int(x) for x in np.asarray(v.flat[1]).ravel()[:3])
    bcol = np.asarray(v.flat[2], np.int32).ravel()
    brow = np.asarray(v.flat[3], np.int32).ravel()
    data = np.asarray(v.flat[4])
    bh = data.shape[0]
    if bh != 64 or data.shape[1] != nb * 64 or bcol.size != nb or brow.size != rows // 64 + 1:
        raise ValueError("BSR cell does not hold 64 x 64 blocks of a %d x %d matrix" % (rows, cols))
    blocks = np.asarray(data, np.float32).T.reshape(nb, 64, 64)  # [j][c][r]
    bits = _f32_to_bf16(blocks).transpose(0, 2, 1)               # [j][r][c]
    return BSRFactor(rows, cols, brow, bcol, bits)


def load(path, ctx=None):
    """Reads a Faust written by ``save`` or by the reference's save_mat_file."""
    import scipy.io as sio
    import scipy.sparse as sps
    from .faust import Faust
    m = sio.loadmat(path, variable_names=[VAR])
    if VAR not in m:
        raise ValueError("%s holds no '%s' variable" % (path, VAR))
    cell = m[VAR]
    if cell.dtype != object or cell.ndim != 2 or cell.shape[0] != 1:
        raise ValueError("'%s' is not a 1 x J cell" % VAR)
    items = list(cell[0])
    if not items:
        raise ValueError("'%s' is empty" % VAR)
    if all(_is_bsr_cell(v) for v in items):
        return Faust([_load_bsr(v) for v in items], ctx=ctx)
    first = items[0]
    if np.iscomplexobj(first.data if sps.issparse(first) else first):
        raise NotImplementedError("complex Fausts are outside the real float32/float64 path")
    dt = np.float32 if (first.dtype == np.float32) else np.float64
    facs = []
    for v in items:
        if _is_bsr_cell(v):
            raise ValueError("a file mixing BSR and CSR factors is not supported")
        s = sps.csr_matrix(v) if sps.issparse(v) else sps.csr_matrix(np.asarray(v))
        facs.append(s.astype(dt))
    return Faust(facs, dtype=dt, ctx=ctx)
