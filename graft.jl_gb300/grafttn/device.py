"""Device context and the tensor-level operations of the library (C ABI calls).

Device tensors are torch complex128 CUDA tensors, used only as allocations: every
arithmetic operation on them goes through libgrafttn (contractions, permutations, QR,
SVD, Krylov solvers).  The context runs on torch's current stream so allocation reuse by
torch's caching allocator is ordered with the library's kernels.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import torch

from . import _lib
from ._lib import check, i64_array, int_array, ptr_array

CDT = torch.complex128


class Context:
    """One library context (device, stream, workspace).  Not shared across threads."""

    def __init__(self, device=0):
        if not torch.cuda.is_available():
            raise RuntimeError("grafttn needs a CUDA device")
        self.device = device
        self.lib = _lib.lib()
        h = C.c_void_p()
        st = self.lib.gtn_ctx_create(device, C.byref(h))
        if st != _lib.GTN_OK:
            raise _lib.GraftError(f"gtn_ctx_create failed with status {st}")
        self.h = h
        with torch.cuda.device(device):
            s = torch.cuda.current_stream(device)
        check(self.lib.gtn_ctx_set_stream(self.h, C.c_void_p(s.cuda_stream)), self.h, "set_stream")
        self.stream = s

    def close(self):
        if self.h:
            self.lib.gtn_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self):
        return int(self.lib.gtn_ctx_launch_count(self.h))

    def sync(self):
        check(self.lib.gtn_ctx_sync(self.h), self.h, "sync")

    def linalg_precision(self, precision=None):
        """The precision of the matrix products inside the factorisations (GTN_PREC_FP64 or
        GTN_PREC_FP64E, gtn_ctx_set_linalg_precision); sets it when given (None leaves it) and
        returns the previous value."""
        old = int(self.lib.gtn_ctx_linalg_precision(self.h))
        if precision is not None:
            prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
            check(self.lib.gtn_ctx_set_linalg_precision(self.h, prec), self.h, "set_linalg_precision")
        return old

    # ---- tensors -------------------------------------------------------------------
    def empty(self, shape):
        return torch.empty(tuple(int(s) for s in shape), dtype=CDT, device=f"cuda:{self.device}")

    def zeros(self, shape):
        """A zero-filled device tensor (gtn_fill)."""
        y = self.empty(shape)
        if y.numel():
            check(self.lib.gtn_fill(self.h, y.numel(), 0.0, 0.0, C.c_void_p(y.data_ptr())), self.h, "fill")
        return y

    def copy_into(self, dst, src):
        """dst <- src (same number of elements, both contiguous) by the library's axpby kernel."""
        if src.numel():
            self.axpby(1.0, src.contiguous().reshape(dst.shape), 0.0, dst)
        return dst

    def copy(self, t):
        """Contiguous copy of a device tensor by the library's axpby kernel (the context
        runs on torch's current stream, so it is ordered with the surrounding work)."""
        t = t.contiguous()
        y = self.empty(t.shape)
        if t.numel():
            self.axpby(1.0, t, 0.0, y)
        return y

    def upload(self, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.complex128))
        return torch.from_numpy(a).to(f"cuda:{self.device}")

    @staticmethod
    def download(t):
        return t.detach().cpu().numpy()

    # ---- operations ----------------------------------------------------------------
    def contract(self, operands, labels, conj=None, order=None, precision=_lib.PREC_FP64):
        """ncon-style contraction of device tensors; returns a new device tensor whose legs
        are ordered -1, -2, ...  (operand 0 starts the pairwise chain)."""
        n = len(operands)
        conj = conj or [False] * n
        order = list(range(n)) if order is None else list(order)
        ranks = [t.dim() for t in operands]
        dims = [int(s) for t in operands for s in t.shape]
        labs = [int(l) for lab in labels for l in lab]
        for t in operands:
            if not t.is_contiguous() or t.dtype != CDT:
                raise ValueError("operands must be contiguous complex128 device tensors")
        outdims = {}
        for t, lab in zip(operands, labels):
            for s, l in zip(t.shape, lab):
                if l < 0:
                    outdims[-l] = int(s)
        out = self.empty([outdims[k] for k in range(1, len(outdims) + 1)])
        st = self.lib.gtn_contract(self.h, n, int_array(ranks), i64_array(dims), int_array(labs),
                                   int_array([1 if c else 0 for c in conj]), int_array(order),
                                   ptr_array([t.data_ptr() for t in operands]), C.c_void_p(out.data_ptr()),
                                   precision)
        check(st, self.h, f"contract {[tuple(t.shape) for t in operands]} labels {labels} order {order}")
        return out

    def contract_vjp(self, operands, labels, ybar, slot, conj=None, order=None, precision=_lib.PREC_FP64):
        """Adjoint of operand `slot` of contract(operands, labels, conj): the tensor G shaped
        like operands[slot] with <G, d op_slot> = <ybar, d y> (gtn_contract_vjp)."""
        n = len(operands)
        conj = conj or [False] * n
        ranks = [t.dim() for t in operands]
        dims = [int(s) for t in operands for s in t.shape]
        labs = [int(l) for lab in labels for l in lab]
        for t in list(operands) + [ybar]:
            if not t.is_contiguous() or t.dtype != CDT:
                raise ValueError("operands must be contiguous complex128 device tensors")
        out = self.empty(tuple(operands[slot].shape))
        st = self.lib.gtn_contract_vjp(self.h, n, int_array(ranks), i64_array(dims), int_array(labs),
                                       int_array([1 if c else 0 for c in conj]),
                                       None if order is None else int_array(order),
                                       ptr_array([t.data_ptr() for t in operands]), slot, C.c_void_p(ybar.data_ptr()),
                                       C.c_void_p(out.data_ptr()), precision)
        check(st, self.h, f"contract_vjp slot {slot} labels {labels}")
        return out

    def tensor_handle(self, t):
        """A gtn_tensor view of the contiguous c128 device tensor t (gtn_tensor_wrap); the
        handle keeps t referenced and is destroyed with the returned object."""
        return TensorHandle(self, t)

    def env_build(self, desc, A, W, envs, precision=_lib.PREC_FP64):
        """env(u->v) from the site description (GTN_MAP_ENV), A_u, W_u and the other
        neighbours' environments (gtn_env_build); returns [ket, op, bra]."""
        hA, hW = TensorHandle(self, A), TensorHandle(self, W)
        he = [TensorHandle(self, e) for e in envs]
        K = desc.n_children
        open_leg = K + 1 if desc.slot < 0 else desc.slot
        wleg = K + 2 if desc.slot < 0 else desc.slot
        out = self.empty((int(A.shape[open_leg]), int(W.shape[wleg]), int(A.shape[open_leg])))
        arr = (C.c_void_p * max(1, len(he)))(*[h.h for h in he])
        check(self.lib.gtn_env_build(self.h, C.byref(desc), hA.h, hW.h, len(he), arr, C.c_void_p(out.data_ptr()),
                                     precision), self.h, "env_build")
        return out

    def restrict_leg(self, t, leg, idx):
        """t with leg `leg` restricted to the indices idx (gtn_restrict_leg, on the device)."""
        t = t.contiguous()
        idx = [int(i) for i in idx]
        shape = list(t.shape)
        shape[leg] = len(idx)
        out = self.empty(tuple(shape))
        check(self.lib.gtn_restrict_leg(self.h, t.dim(), i64_array([int(s) for s in t.shape]), leg, len(idx),
                                        i64_array(idx), C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr())),
              self.h, "restrict_leg")
        return out

    def permute(self, t, perm):
        if t.dim() == 0:
            return self.copy(t)
        out = self.empty([t.shape[p] for p in perm])
        st = self.lib.gtn_permute(self.h, t.dim(), i64_array([int(s) for s in t.shape]), int_array(perm),
                                  C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()))
        check(st, self.h, "permute")
        return out

    def qr(self, A2):
        """Thin QR of a row-major m x n device matrix: (Q m x k, R k x n)."""
        m, n = A2.shape
        k = min(m, n)
        Q = self.empty((m, k))
        R = self.empty((k, n))
        check(self.lib.gtn_qr(self.h, m, n, C.c_void_p(A2.data_ptr()), C.c_void_p(Q.data_ptr()),
                              C.c_void_p(R.data_ptr())), self.h, "qr")
        return Q, R

    def svd_trunc(self, A2, maxdim=None, atol=0.0, rtol=0.0, discarded_weight=0.0):
        m, n = A2.shape
        k = min(m, n)
        U = self.empty((m * k,))
        Vh = self.empty((k * n,))
        S = (C.c_double * k)()
        rank = C.c_int64()
        disc = C.c_double()
        st = self.lib.gtn_svd_trunc(self.h, m, n, C.c_void_p(A2.data_ptr()), int(maxdim or 0), float(atol),
                                    float(rtol), float(discarded_weight), C.c_void_p(U.data_ptr()), S,
                                    C.c_void_p(Vh.data_ptr()), C.byref(rank), C.byref(disc))
        check(st, self.h, "svd_trunc")
        r = rank.value
        return U[: m * r].view(m, r), np.array(S[:r]), Vh[: r * n].view(r, n), disc.value

    def diag_scale(self, A2, d, side=0):
        """In place: side 0 scales columns (A diag(d)), side 1 scales rows (diag(d) A)."""
        rows, cols = A2.shape
        arr = (C.c_double * len(d))(*[float(v) for v in d])
        check(self.lib.gtn_diag_scale(self.h, rows, cols, arr, side, C.c_void_p(A2.data_ptr())), self.h,
              "diag_scale")
        return A2

    def matmul(self, A, B, conjA=False, transA=False):
        """op(A) @ B for row-major device matrices, op = conj and / or transpose (FP64
        contraction; B starts the chain so that the conjugated operand is a static)."""
        la = [1, -1] if transA else [-1, 1]
        return self.contract([B.contiguous(), A.contiguous()], [[1, -2], la], [False, conjA])

    def concat_cols(self, A, B):
        """[A B] for row-major matrices with equal row counts."""
        rows = A.shape[0]
        out = self.empty((rows, A.shape[1] + B.shape[1]))
        ld = out.shape[1]
        check(self.lib.gtn_copy2d(self.h, rows, A.shape[1], C.c_void_p(A.data_ptr()), A.shape[1],
                                  C.c_void_p(out.data_ptr()), ld), self.h, "copy2d")
        if B.shape[1]:
            check(self.lib.gtn_copy2d(self.h, rows, B.shape[1], C.c_void_p(B.data_ptr()), B.shape[1],
                                      C.c_void_p(out.data_ptr() + 16 * A.shape[1]), ld), self.h, "copy2d")
        return out

    def dot(self, x, y):
        out = (C.c_double * 2)()
        check(self.lib.gtn_dot(self.h, x.numel(), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), out),
              self.h, "dot")
        return complex(out[0], out[1])

    def axpby(self, a, x, b, y):
        a, b = complex(a), complex(b)
        check(self.lib.gtn_axpby(self.h, x.numel(), a.real, a.imag, C.c_void_p(x.data_ptr()), b.real, b.imag,
                                 C.c_void_p(y.data_ptr())), self.h, "axpby")
        return y

    def scale(self, x, a):
        """New tensor a * x."""
        y = self.empty(x.shape)
        return self.axpby(a, x, 0.0, y)

    def norm(self, x):
        return float(np.sqrt(max(self.dot(x, x).real, 0.0)))


_DEFAULT = {}
_LOCK = threading.Lock()


def default_context(device=0):
    with _LOCK:
        ctx = _DEFAULT.get((threading.get_ident(), device))
        if ctx is None:
            ctx = Context(device)
            _DEFAULT[(threading.get_ident(), device)] = ctx
        return ctx


class TensorHandle:
    """gtn_tensor view of a device tensor (no copy)."""

    def __init__(self, ctx, t):
        if not t.is_contiguous() or t.dtype != CDT:
            raise ValueError("tensor handles need contiguous complex128 device tensors")
        self.ctx, self.t = ctx, t
        h = C.c_void_p()
        check(ctx.lib.gtn_tensor_wrap(ctx.h, t.dim(), i64_array([int(x) for x in t.shape]), C.c_void_p(t.data_ptr()),
                                      C.byref(h)), ctx.h, "tensor_wrap")
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.ctx.lib.gtn_tensor_destroy(self.h)
                self.h = None
        except Exception:
            pass
