"""Python mirror of FAuST's Faust (pyfaust.Faust / Faust::TransformHelper)
over the C ABI.

A Faust is a product of sparse factors S_0 ... S_{J-1}; ``F @ X`` applies
them right to left like TransformHelper<FPP,Cpu>::multiply
(src/faust_linear_operator/CPU/faust_TransformHelper.hpp:340-433) and
pyfaust.Faust.__matmul__ (wrapper/python/pyfaust.py:1092-1203).  Factors live
in device memory; the product runs on the GPU only.
"""
import ctypes

import numpy as np

from . import _ffi
from ._ffi import check


def _np_dtype_code(dt):
    dt = np.dtype(dt)
    if dt == np.float64:
        return _ffi.F64
    if dt == np.float32:
        return _ffi.F32
    raise TypeError("CSR Fausts are float32 or float64 (got %s)" % dt)


class Context:
    """A device + stream pair (fgb_ctx); one per host thread."""

    def __init__(self, device=0, stream=None):
        """stream: a cudaStream_t handle (int); by default torch's current
        stream on that device, so that work is ordered with torch's."""
        if stream is None:
            try:
                import torch
                if torch.cuda.is_available():
                    stream = torch.cuda.current_stream(device).cuda_stream
            except ImportError:
                pass
        h = ctypes.c_void_p()
        check(_ffi.lib().fgb_ctx_create(int(device), ctypes.c_void_p(stream or 0), ctypes.byref(h)))
        self.stream = stream or 0
        self.handle = h
        self.device = device

    def synchronize(self):
        check(_ffi.lib().fgb_ctx_synchronize(self.handle), self.handle)

    def cancel(self):
        check(_ffi.lib().fgb_cancel(self.handle), self.handle)

    def kernel_launches(self):
        return int(_ffi.lib().fgb_ctx_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            _ffi.lib().fgb_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = {}


def default_context(device=0):
    if device not in _default:
        _default[device] = Context(device)
    return _default[device]


class BSRFactor:
    """A BSR factor with 64 x 64 BF16 blocks (MatBSR, faust_MatBSR.h:41-145).

    browptr: (rows/64+1,) int32; bcolind: (nblocks,) int32; blocks:
    (nblocks, 64, 64) block values, C-ordered as block[i][r][c] (converted
    here to the column-major block storage of BSRMat)."""

    def __init__(self, rows, cols, browptr, bcolind, blocks_bf16_bits):
        self.shape = (int(rows), int(cols))
        self.browptr = np.ascontiguousarray(browptr, np.int32)
        self.bcolind = np.ascontiguousarray(bcolind, np.int32)
        b = np.asarray(blocks_bf16_bits, np.uint16)
        assert b.ndim == 3 and b.shape[1] == 64 and b.shape[2] == 64
        # column-major per block: element (r, c) at c*64 + r
        self.blocks_colmajor = np.ascontiguousarray(b.transpose(0, 2, 1))

    @property
    def nnz_blocks(self):
        return int(self.bcolind.size)


def _order_code(order):
    codes = {"DEFAULT_L2R": _ffi.ORDER_DEFAULT_L2R, "DYNPROG": _ffi.ORDER_DYNPROG}
    if isinstance(order, str):
        if order.upper() not in codes:
            raise ValueError("order must be DEFAULT_L2R or DYNPROG")
        return codes[order.upper()]
    return int(order)


def _torch_dtype(dt):
    import torch
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}[np.dtype(dt)]


def dynprog_plan(leaves, op="N"):
    """Split table of the library's DYNPROG (host code, no device):
    leaves = [(rows, cols, nnz, is_dense)]; returns {(i, j): k}."""
    n = len(leaves)
    a = np.asarray(leaves, np.int64).reshape(n, 4)
    rows, cols, nnz, dense = (np.ascontiguousarray(a[:, q], np.int32) for q in range(4))
    split = np.zeros(n * n, np.int32)
    rc = _ffi.lib().fgb_dynprog_plan(n, rows.ctypes.data, cols.ctypes.data, nnz.ctypes.data, dense.ctypes.data,
                                     op.upper().encode(), split.ctypes.data)
    if rc != 0:
        raise ValueError("fgb_dynprog_plan failed (%d)" % rc)
    return {(i, j): int(split[i * n + j]) for i in range(n) for j in range(i + 1, n)}


def _is_colmajor(T):
    rows, cols = T.shape
    return (T.stride(0) == 1 or rows == 1) and (cols == 1 or T.stride(1) >= rows)


def _ld(T):
    """Leading dimension of a column-major tensor (any value >= rows works
    for a single column)."""
    return T.stride(1) if T.shape[1] > 1 else max(1, T.shape[0])


def _csr_desc(m, keep):
    import scipy.sparse as sp
    m = sp.csr_matrix(m)
    m.sort_indices()
    rp = np.ascontiguousarray(m.indptr, np.int32)
    ci = np.ascontiguousarray(m.indices, np.int32)
    keep += [rp, ci]
    return rp, ci, m


class Faust:
    """Device-resident product of CSR (float32/float64) or BSR (bf16) factors."""

    def __init__(self, factors, dtype=None, ctx=None):
        self.ctx = ctx or default_context()
        keep = []
        descs = (_ffi.FactorDesc * len(factors))()
        if all(isinstance(f, BSRFactor) for f in factors):
            self.dtype_code = _ffi.BF16
            self.dtype = "bfloat16"
            for i, f in enumerate(factors):
                keep += [f.browptr, f.bcolind, f.blocks_colmajor]
                descs[i] = _ffi.FactorDesc(_ffi.BSR, f.shape[0], f.shape[1], f.nnz_blocks, 64, 64,
                                           f.browptr.ctypes.data, f.bcolind.ctypes.data,
                                           f.blocks_colmajor.ctypes.data)
        else:
            dt = np.dtype(dtype or factors[0].dtype)
            self.dtype_code = _np_dtype_code(dt)
            self.dtype = dt
            for i, f in enumerate(factors):
                rp, ci, m = _csr_desc(f, keep)
                v = np.ascontiguousarray(m.data, dt)
                keep.append(v)
                descs[i] = _ffi.FactorDesc(_ffi.CSR, m.shape[0], m.shape[1], m.nnz, 0, 0, rp.ctypes.data,
                                           ci.ctypes.data, v.ctypes.data)
        h = ctypes.c_void_p()
        check(_ffi.lib().fgb_faust_create(self.ctx.handle, self.dtype_code, len(factors), descs, ctypes.byref(h)),
              self.ctx.handle)
        self.handle = h
        r, c, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ffi.lib().fgb_faust_shape(h, ctypes.byref(r), ctypes.byref(c), ctypes.byref(n))
        self.shape = (r.value, c.value)
        self._n = n.value

    @classmethod
    def _from_handle(cls, handle, ctx, dtype):
        self = cls.__new__(cls)
        self.ctx = ctx
        self.handle = handle
        self.dtype = np.dtype(dtype)
        self.dtype_code = _np_dtype_code(self.dtype)
        r, c, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ffi.lib().fgb_faust_shape(handle, ctypes.byref(r), ctypes.byref(c), ctypes.byref(n))
        self.shape = (r.value, c.value)
        self._n = n.value
        return self

    def numfactors(self):
        return self._n

    def __len__(self):
        return self._n

    # -- products ---------------------------------------------------------
    def __matmul__(self, X):
        """F @ X for a host numpy array (host entry point) or a CUDA tensor."""
        if hasattr(X, "is_cuda") and X.is_cuda:
            return self.matmul_device(X)
        X = np.asfortranarray(X, dtype=self.dtype)
        if X.ndim != 2 or X.shape[0] != self.shape[1]:
            raise ValueError("dimensions do not match: Faust %s @ %s" % (self.shape, X.shape))
        Y = np.zeros((self.shape[0], X.shape[1]), dtype=self.dtype, order="F")
        check(_ffi.lib().fgb_faust_mul_host(self.handle, X.ctypes.data, X.shape[1], Y.ctypes.data), self.ctx.handle)
        return Y

    def matmul_device(self, X, Y=None, mode=0):
        """Y = F X with column-major CUDA tensors (X given as a (ncols, rows)
        row-major tensor is the same memory as a column-major (rows, ncols)
        matrix: pass X.t() views or use colmajor tensors from faust_gb300.synth)."""
        import torch
        Xc = X
        rows_in, ncols = self.shape[1], X.shape[1]
        if X.shape[0] != rows_in:
            raise ValueError("dimensions do not match")
        # column-major storage = transpose of a contiguous (ncols, rows) tensor
        if not _is_colmajor(X):
            Xc = X.t().contiguous().t()
        if Y is None:
            Y = torch.empty((ncols, self.shape[0]), dtype=X.dtype, device=X.device).t()
        elif not _is_colmajor(Y):
            raise ValueError("Y must be column-major")
        check(_ffi.lib().fgb_faust_mul(self.handle, Xc.data_ptr(), _ld(Xc), ncols, Y.data_ptr(), _ld(Y), int(mode)),
              self.ctx.handle)
        return Y

    def matmul_op_device(self, op, X, Y=None, mode=0):
        """Y = op(F) X on the device with op in 'N', 'T', 'H' (H = T for real
        scalars): Transform::multiply(X, op).  Column-major CUDA tensors."""
        import torch
        op = op.upper()
        if op == "N":
            return self.matmul_device(X, Y, mode)
        rows_in, rows_out, ncols = self.shape[0], self.shape[1], X.shape[1]
        if X.shape[0] != rows_in:
            raise ValueError("dimensions do not match: %s(F) with F %s @ %s" % (op, self.shape, tuple(X.shape)))
        Xc = X if _is_colmajor(X) else X.t().contiguous().t()
        if Y is None:
            Y = torch.empty((ncols, rows_out), dtype=X.dtype, device=X.device).t()
        elif not _is_colmajor(Y):
            raise ValueError("Y must be column-major")
        check(_ffi.lib().fgb_faust_mul_op(self.handle, op.encode(), Xc.data_ptr(), _ld(Xc), ncols, Y.data_ptr(),
                                          _ld(Y), int(mode)), self.ctx.handle)
        return Y

    def product_device(self, op="N", order="DEFAULT_L2R", Y=None):
        """Dense op(F) on the device (TransformHelper::get_product): order
        'DEFAULT_L2R' (Transform::get_product) or 'DYNPROG' (dynprog_multiply).
        Returns a column-major CUDA tensor."""
        import torch
        op = op.upper()
        code = _order_code(order)
        rows, cols = self.shape if op == "N" else self.shape[::-1]
        if Y is None:
            Y = torch.empty((cols, rows), dtype=_torch_dtype(self.dtype), device="cuda:%d" % self.ctx.device).t()
        elif not _is_colmajor(Y) or tuple(Y.shape) != (rows, cols):
            raise ValueError("Y must be a column-major %d x %d tensor" % (rows, cols))
        check(_ffi.lib().fgb_faust_product(self.handle, op.encode(), code, Y.data_ptr(), _ld(Y)), self.ctx.handle)
        return Y

    def matmul_dynprog_device(self, X, op="N", Y=None):
        """Y = op(F) X with the product order chosen by DYNPROG
        (TransformHelper::multiply with mul_order_opt_mode DYNPROG)."""
        import torch
        op = op.upper()
        rows_in, rows_out = (self.shape[1], self.shape[0]) if op == "N" else self.shape
        if X.shape[0] != rows_in:
            raise ValueError("dimensions do not match: %s(F) with F %s @ %s" % (op, self.shape, tuple(X.shape)))
        Xc = X if _is_colmajor(X) else X.t().contiguous().t()
        ncols = X.shape[1]
        if Y is None:
            Y = torch.empty((ncols, rows_out), dtype=X.dtype, device=X.device).t()
        elif not _is_colmajor(Y):
            raise ValueError("Y must be column-major")
        check(_ffi.lib().fgb_faust_mul_dynprog(self.handle, op.encode(), Xc.data_ptr(), _ld(Xc), ncols, Y.data_ptr(),
                                               _ld(Y)), self.ctx.handle)
        return Y

    def norm(self, ord=2, max_iter=100, threshold=1e-6):
        """2-norm by FP64 power iteration (TransformHelper::spectralNorm)."""
        if ord != 2:
            raise NotImplementedError("only the 2-norm runs on the GPU path")
        out, flag = ctypes.c_double(), ctypes.c_int()
        check(_ffi.lib().fgb_faust_spectral_norm(self.handle, int(max_iter), float(threshold), ctypes.byref(out),
                                                 ctypes.byref(flag)), self.ctx.handle)
        return out.value

    def factors(self, i):
        """Factor i as a scipy CSR matrix (copied to host)."""
        import scipy.sparse as sp
        fmt, r, c, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(_ffi.lib().fgb_faust_factor_info(self.handle, int(i), ctypes.byref(fmt), ctypes.byref(r),
                                               ctypes.byref(c), ctypes.byref(nnz)), self.ctx.handle)
        rp = np.zeros(r.value + 1, np.int32)
        ci = np.zeros(max(1, nnz.value), np.int32)
        v = np.zeros(max(1, nnz.value), self.dtype)
        check(_ffi.lib().fgb_faust_factor_to_csr(self.handle, int(i), rp.ctypes.data, ci.ctypes.data, v.ctypes.data),
              self.ctx.handle)
        return sp.csr_matrix((v[:nnz.value], ci[:nnz.value], rp), shape=(r.value, c.value))

    def bsr_factor(self, i):
        """Factor i of a BF16 Faust as a BSRFactor (copied to host)."""
        fmt, r, c, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(_ffi.lib().fgb_faust_factor_info(self.handle, int(i), ctypes.byref(fmt), ctypes.byref(r),
                                               ctypes.byref(c), ctypes.byref(nb)), self.ctx.handle)
        if fmt.value != _ffi.BSR:
            raise ValueError("factor %d is not BSR" % i)
        brow = np.zeros(r.value // 64 + 1, np.int32)
        bcol = np.zeros(max(1, nb.value), np.int32)
        blocks = np.zeros((max(1, nb.value), 64, 64), np.uint16)  # [j][c][r]: column-major blocks
        check(_ffi.lib().fgb_faust_factor_to_bsr(self.handle, int(i), brow.ctypes.data, bcol.ctypes.data,
                                                 blocks.ctypes.data), self.ctx.handle)
        n = nb.value
        return BSRFactor(r.value, c.value, brow, bcol[:n], blocks[:n].transpose(0, 2, 1))

    def save(self, filepath, format="Matlab"):
        """Writes the Faust as a MAT5 file (Faust.save / Transform::save_mat_file,
        faust_Transform.hpp:434-475): variable 'faust_factors', a 1 x J cell."""
        if format != "Matlab":
            raise ValueError("only the Matlab (.mat) format is supported")
        from . import matio
        matio.save(self, filepath)

    @staticmethod
    def load(filepath, ctx=None):
        """Reads a Faust from a .mat file (Transform::read_from_mat_file,
        faust_Transform.hpp:481-514)."""
        from . import matio
        return matio.load(filepath, ctx)

    def toarray(self, order="DEFAULT_L2R"):
        """Full product as a host array (pyfaust Faust.toarray: get_product).
        BF16 BSR Fausts: F applied to the identity."""
        if self.dtype_code == _ffi.BF16:
            return self @ np.eye(self.shape[1], dtype=self.dtype)
        Y = self.product_device("N", order)
        self.ctx.synchronize()
        return Y.cpu().numpy()

    def close(self):
        if getattr(self, "handle", None):
            _ffi.lib().fgb_faust_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
