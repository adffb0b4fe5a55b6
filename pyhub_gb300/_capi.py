"""Typed ctypes bindings of include/pyhub_ed.h and a thin device-side sector
object.  Vectors are torch CUDA tensors; only their data pointers cross the
C ABI.  Every call checks the status code and raises ``EDError`` with the
library's message."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from .libs import libcore

ED_OK, ED_ERR_ARG, ED_ERR_CUDA, ED_ERR_MEM, ED_ERR_RANGE = 0, 1, 2, 3, 4
ED_HUBBARD, ED_HEISENBERG = 0, 1
ED_F32, ED_F64 = 0, 1

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double

_SIGS = {
    "ed_last_error": (ctypes.c_char_p, []),
    "ed_version": (_I, []),
    "ed_binom": (_I64, [_I, _I]),
    "ed_basis": (_I, [_I, _I, _P, _I64]),
    "ed_rank": (_I64, [_I, _I, ctypes.c_uint32]),
    "ed_sector_create": (_I, [_I, _I, _I, _I, _P, _P, _P, ctypes.POINTER(_P)]),
    "ed_sector_destroy": (_I, [_P]),
    "ed_lanczos_step_scratch_bytes": (_I64, [_P, _I]),
    "ed_lanczos_step": (_I, [_P, _P, _I, _I64, _P, _I64, _I, _I, _P, _P, _P, _P, _P, _I64]),
    "ed_rdm1_scratch_bytes": (_I64, [_P]),
    "ed_rdm1": (_I, [_P, _P, _I, _I64, _P, _P, _P, _P, _P, _I64]),
    "ed_hf_grad": (_I, [_P, _P, _I, _I64, _P, _I, _P, _P, _P, _P, _P, _I64]),
    "ed_opspace_create": (_I, [_I, _I, _P, _I, _P, ctypes.POINTER(_P)]),
    "ed_opspace_dims": (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "ed_opspace_destroy": (_I, [_P]),
    "ed_ops_apply": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _P, _I64]),
    "ed_sector_dims": (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "ed_sector_strings": (_I, [_P, _P, _P]),
    "ed_sector_nnz": (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "ed_scratch_bytes": (_I64, [_I64, _I]),
    "ed_hv": (_I, [_P, _P, _I, _I64, _P, _P, _D, _P, _P, _I64]),
    "ed_multidot": (_I, [_P, _I, _I64, _P, _I64, _I, _P, _P, _P, _P, _I64]),
    "ed_update": (_I, [_P, _I, _I, _I64, _P, _I64, _I, _P, _P, _P, _P, _P, _I64]),
    "ed_rdm_scratch_bytes": (_I64, [_I]),
    "ed_rdm": (_I, [_P, _P, _I, _I64, _P, _P, _I, _P, _I, _P, _P, _I64]),
    "ed_gf_start": (_I, [_P, _P, _P, _I, _I, _I, _I64, _P, _I, _I64, _P]),
    "ed_batch_create": (_I, [_I, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "ed_batch_destroy": (_I, [_P]),
    "ed_batch_layout": (_I, [_P, ctypes.POINTER(_I64), _P, _P, ctypes.POINTER(_I64)]),
    "ed_batch_scratch_bytes": (_I64, [_P]),
    "ed_batch_lanczos": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _I64]),
    "ed_batch_hv": (_I, [_P, _P, _I, _P, _P, _P, _I64]),
    "ed_sector_set_uijkl": (_I, [_P, _P]),
    "ed_batch_lanczos_persistent": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _P, _I64]),
    "ed_batch_persistent_status": (_I, [_P, _P, ctypes.POINTER(_I)]),
    "ed_batch_persistent_watchdog": (_I, [_P, ctypes.c_double, _I]),
    "ed_dbl_occ_scratch_bytes": (_I64, [_P, _I]),
    "ed_dbl_occ": (_I, [_P, _P, _I, _I64, _P, _P, _I, _P, _P, _P, _I64]),
    "ed_batch_ritz": (_I, [_P, _P, _I, _P, _P, _I, _P, _P, _P, _P, _P, _I64]),
    "ed_batch_create_rows": (_I, [_I, _P, _I, ctypes.POINTER(_P)]),
    "ed_batch_rows": (_I, [_P]),
    "ed_update_wscaled": (_I, [_P, _I, _I, _I64, _P, _I64, _I, _P, _P, _P, _P, _P, _P, _I64]),
    "ed_lanczos_state_doubles": (_I64, [_I]),
    "ed_batch_lanczos_kept": (_I, [_P, _P, _I, _P, _P, _P, _I, _P, _P, _P, _I64]),
    "ed_batch_ritz_sum": (_I, [_P, _P, _I, _P, _I, _P, _P, _P]),
    "ed_cf_eval": (_I, [_P, _I, _I, _P, _P, _I, _P, _P, _P, _P]),
    "ed_gf_start_sites": (_I, [_P, _P, _P, _I, _I, _P, _I, _I64, _P, _I, _I64, _P, _I64]),
    "ed_lanczos_coef": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P]),
}

GF_KINDS = {"h_up": 0, "h_down": 1, "e_up": 2, "e_down": 3}

_bound = None


class EDError(RuntimeError):
    """A nonzero status from the C ABI."""

    def __init__(self, func: str, code: int, msg: str):
        super().__init__(f"{func} failed with status {code}: {msg}")
        self.code = code


def lib():
    global _bound
    if _bound is None:
        L = libcore()
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _bound = L
    return _bound


def check(func: str, rc: int):
    if rc != ED_OK:
        raise EDError(func, rc, lib().ed_last_error().decode(errors="replace"))


def _ptr(t, need: int | None = None, what: str = "tensor") -> int | None:
    """Device pointer of a tensor handed to a kernel.  Refuses what would make
    a kernel read or write outside the caller's memory: host tensors, a
    non-unit innermost stride, and (with ``need``) fewer than ``need``
    elements."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor (got device {t.device})")
    if t.dim() > 0 and t.stride(-1) != 1:
        raise ValueError(f"{what} must have unit stride in its last dimension")
    if need is not None and t.numel() < need:
        raise ValueError(f"{what} holds {t.numel()} elements, {need} needed")
    return t.data_ptr()


def _stream(stream) -> int | None:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream if isinstance(stream, int) else stream.cuda_stream


def dtype_code(dt) -> int:
    import torch
    if dt == torch.float32:
        return ED_F32
    if dt == torch.float64:
        return ED_F64
    raise TypeError(f"unsupported vector dtype {dt}")


# ------------------------------------------------------------------ basis ---

def binom(n: int, k: int) -> int:
    return int(lib().ed_binom(n, k))


def basis(norb: int, ne: int) -> np.ndarray:
    """Spin strings in the reference order (compute_basis.f90:67-96)."""
    n = binom(norb, ne)
    out = np.zeros(max(n, 1), dtype=np.uint32)
    check("ed_basis", lib().ed_basis(norb, ne, out.ctypes.data, n))
    return out[:n]


def rank(norb: int, ne: int, s: int) -> int:
    return int(lib().ed_rank(norb, ne, int(s) & 0xFFFFFFFF))


def scratch_bytes(n: int, nvec: int) -> int:
    return int(lib().ed_scratch_bytes(int(n), int(nvec)))


# ----------------------------------------------------------------- sector ---

@dataclass
class Dims:
    nsup: int
    nsdn: int
    dim: int


class Sector:
    """Device tables of one (norb, nup, ndn) sector; owns an ed_sector*.

    Vectors in the internal layout are [nsdn, ld] with ld = nsup rounded up
    to a multiple of 32 (zero padding); ``to_ref``/``from_ref`` convert to the
    reference's flat index d*nsup+u."""

    PAD = 32

    def __init__(self, norb: int, nup: int, ndn: int, kind: int = ED_HUBBARD, t=None, U=None, J=None):
        self.norb, self.nup, self.ndn, self.kind = int(norb), int(nup), int(ndn), kind
        h = _P()
        tt = None if t is None else np.ascontiguousarray(t, dtype=np.float64).reshape(norb, norb)
        uu = None if U is None else np.ascontiguousarray(np.broadcast_to(np.asarray(U, dtype=np.float64), (norb,)))
        jj = None if J is None else np.ascontiguousarray(J, dtype=np.float64).reshape(norb, norb)
        self._keep = (tt, uu, jj)
        check("ed_sector_create", lib().ed_sector_create(
            self.norb, self.nup, self.ndn, kind,
            None if tt is None else tt.ctypes.data, None if uu is None else uu.ctypes.data,
            None if jj is None else jj.ctypes.data, ctypes.byref(h)))
        self._h = h
        a, b, c = _I64(), _I64(), _I64()
        check("ed_sector_dims", lib().ed_sector_dims(h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        self.nsup, self.nsdn, self.dim = a.value, b.value, c.value
        if kind == ED_HUBBARD:
            self.ld = (self.nsup + self.PAD - 1) // self.PAD * self.PAD
            self.n = self.nsdn * self.ld
        else:
            self.ld = self.nsup
            self.n = (self.nsup + self.PAD - 1) // self.PAD * self.PAD

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ed_sector_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def strings(self):
        up = np.zeros(max(self.nsup, 1), dtype=np.uint32)
        dn = np.zeros(max(self.nsdn, 1), dtype=np.uint32)
        check("ed_sector_strings", lib().ed_sector_strings(self._h, up.ctypes.data, dn.ctypes.data))
        return up[:self.nsup], dn[:self.nsdn]

    def nnz(self):
        a, b = _I64(), _I64()
        check("ed_sector_nnz", lib().ed_sector_nnz(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # -------------------------------------------------------- layouts
    def zeros(self, dtype, device=None, *shape):
        import torch
        return torch.zeros(*shape, self.n, dtype=dtype, device=device or "cuda")

    def to_ref(self, v):
        """Internal layout -> reference flat layout (a view when ld == nsup)."""
        if self.kind == ED_HUBBARD:
            return v.view(*v.shape[:-1], self.nsdn, self.ld)[..., : self.nsup].reshape(*v.shape[:-1], self.dim)
        return v[..., : self.dim]

    def from_ref(self, r, out=None):
        import torch
        if out is None:
            out = torch.zeros(*r.shape[:-1], self.n, dtype=r.dtype, device=r.device)
        if self.kind == ED_HUBBARD:
            out.view(*r.shape[:-1], self.nsdn, self.ld)[..., : self.nsup] = r.reshape(*r.shape[:-1], self.nsdn, self.nsup)
        else:
            out[..., : self.dim] = r
        return out

    # -------------------------------------------------------- composite entry points
    def rdm1(self, psi, ld: int | None = None, stream=None):
        """ed_rdm1: (gamma [2, N, N], docc [N], sisj [N, N]) as the reference
        stores them (Heisenberg: gamma and docc are None)."""
        import torch
        N = self.norb
        nb = int(lib().ed_rdm1_scratch_bytes(self._h))
        scratch = torch.empty((nb + 7) // 8, dtype=torch.float64, device=psi.device)
        hub = self.kind == ED_HUBBARD
        gamma = np.zeros((2, N, N)) if hub else None
        docc = np.zeros(N) if hub else None
        sisj = np.zeros((N, N))
        ld = self.ld if ld is None else ld
        check("ed_rdm1", lib().ed_rdm1(self._h, _stream(stream), dtype_code(psi.dtype), int(ld),
                                       _ptr(psi, self._need(ld), "psi"),
                                       None if gamma is None else gamma.ctypes.data,
                                       None if docc is None else docc.ctypes.data, sisj.ctypes.data,
                                       _ptr(scratch), nb))
        return gamma, docc, sisj

    def hf_grad(self, psi, bonds, ld: int | None = None, stream=None):
        """ed_hf_grad: (g_t [nbonds], g_u [N], g_eps [N]) of <psi|H|psi>; bonds
        1-based (i, j) pairs."""
        import torch
        N = self.norb
        b = np.ascontiguousarray(np.asarray(bonds, dtype=np.int32).reshape(-1, 2))
        nb = int(lib().ed_rdm1_scratch_bytes(self._h))
        scratch = torch.empty((nb + 7) // 8, dtype=torch.float64, device=psi.device)
        gt, gu, ge = np.zeros(max(len(b), 1)), np.zeros(N), np.zeros(N)
        ld = self.ld if ld is None else ld
        check("ed_hf_grad", lib().ed_hf_grad(self._h, _stream(stream), dtype_code(psi.dtype), int(ld),
                                             _ptr(psi, self._need(ld), "psi"), len(b), b.ctypes.data,
                                             gt.ctypes.data, gu.ctypes.data, ge.ctypes.data, _ptr(scratch), nb))
        return gt[:len(b)], gu, ge

    def lanczos_step(self, V, k: int, mmax: int, w, state, alpha, beta, scratch, ld: int | None = None,
                     stream=None):
        """ed_lanczos_step: step k of the full-reorthogonalisation Lanczos on the
        basis rows V (device [mmax+1, n]); scratch as ed_lanczos_step_scratch_bytes,
        the same for every step of a run."""
        ld = self.ld if ld is None else ld
        check("ed_lanczos_step", lib().ed_lanczos_step(
            self._h, _stream(stream), dtype_code(V.dtype), int(ld), _ptr(V), int(V.stride(0)), int(k), int(mmax),
            _ptr(w), _ptr(state), _ptr(alpha), _ptr(beta), _ptr(scratch),
            int(scratch.numel() * scratch.element_size())))

    def lanczos_step_scratch_bytes(self, mmax: int) -> int:
        return int(lib().ed_lanczos_step_scratch_bytes(self._h, int(mmax)))

    # -------------------------------------------------------- products
    def rdm_raw(self, bra, ket=None, pairs=None, flags: int = 3, ld: int | None = None, stream=None):
        """Raw per-pair sums of ed_rdm as a host float64 array
        ([npairs, 6] for Hubbard, [npairs, 2] for Heisenberg) and the pair list."""
        import torch
        ket = bra if ket is None else ket
        if pairs is None:
            pairs = [(J, K) for J in range(1, self.norb + 1) for K in range(1, self.norb + 1)]
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        npairs = len(pr)
        nq = 6 if self.kind == ED_HUBBARD else 2
        out = torch.zeros(nq * npairs, dtype=torch.float64, device=bra.device)
        nb = int(lib().ed_rdm_scratch_bytes(npairs))
        scratch = torch.empty((nb + 7) // 8, dtype=torch.float64, device=bra.device)
        ld = self.ld if ld is None else ld
        need = self._need(ld)
        if ket.dtype != bra.dtype:
            raise TypeError("bra and ket must have the same dtype")
        check("ed_rdm", lib().ed_rdm(self._h, _stream(stream), dtype_code(bra.dtype), int(ld), _ptr(bra, need, "bra"),
                                     _ptr(ket, need, "ket"), npairs, pr.ctypes.data, int(flags), _ptr(out),
                                     _ptr(scratch), nb))
        o = out.cpu().numpy()
        if self.kind == ED_HUBBARD:
            raw = np.concatenate([o[: 4 * npairs].reshape(npairs, 4), o[4 * npairs:].reshape(npairs, 2)], axis=1)
        else:
            raw = o.reshape(npairs, 2)
        return raw, pr

    def set_uijkl(self, Ul):
        """Add the U_ijkl interaction (the reference's is_Uloc=3 path): Ul is
        the (norb,)*4 tensor as FermiHubbard takes it; the on-site U is dropped."""
        u = np.ascontiguousarray(Ul, dtype=np.float64).reshape((self.norb,) * 4)
        self._keep = self._keep + (u,)
        check("ed_sector_set_uijkl", lib().ed_sector_set_uijkl(self._h, u.ctypes.data))

    def dbl_occ(self, bra, ket=None, quads=None, ld: int | None = None, stream=None):
        """DBL_OCC(J,K,M,N) = <ket|c+_{K up} c_{J up} c+_{N down} c_{M down}|bra>
        for the given 1-based quads ([n][4]); returns (host FP64 [n], quads)."""
        import torch
        ket = bra if ket is None else ket
        q = np.ascontiguousarray(np.asarray(quads, dtype=np.int32).reshape(-1, 4))
        out = torch.zeros(len(q), dtype=torch.float64, device=bra.device)
        nb = int(lib().ed_dbl_occ_scratch_bytes(self._h, len(q)))
        scratch = torch.empty((nb + 7) // 8, dtype=torch.float64, device=bra.device)
        ld = self.ld if ld is None else ld
        need = self._need(ld)
        if ket.dtype != bra.dtype:
            raise TypeError("bra and ket must have the same dtype")
        check("ed_dbl_occ", lib().ed_dbl_occ(self._h, _stream(stream), dtype_code(bra.dtype), int(ld),
                                             _ptr(bra, need, "bra"), _ptr(ket, need, "ket"), len(q), q.ctypes.data,
                                             _ptr(out), _ptr(scratch), nb))
        return out.cpu().numpy(), q

    def hv(self, x, y, scale: float = 1.0, dots=None, scratch=None, ld: int | None = None, stream=None):
        """y = scale * H x (device tensors in the internal layout unless ld is given)."""
        ld = self.ld if ld is None else ld
        sb = 0 if scratch is None else scratch.numel() * scratch.element_size()
        need = self._need(ld)
        if y.dtype != x.dtype:
            raise TypeError("x and y must have the same dtype")
        check("ed_hv", lib().ed_hv(self._h, _stream(stream), dtype_code(x.dtype), int(ld), _ptr(x, need, "x"),
                                   _ptr(y, need, "y"), float(scale), _ptr(dots, 2, "dots"), _ptr(scratch),
                                   int(sb)))

    def _need(self, ld: int) -> int:
        """Elements a vector with row stride ld must hold."""
        if self.kind != ED_HUBBARD:
            return self.dim
        return (self.nsdn - 1) * int(ld) + self.nsup if self.nsdn > 0 else 0


class OpSpace:
    """ed_opspace: the vector space of the generic operator engine (every
    listed up-particle number times every listed down-particle number,
    state (d, u) at d*nsup + u)."""

    def __init__(self, norb: int, nups, ndns):
        self.norb = int(norb)
        nu = np.ascontiguousarray(np.asarray(list(nups), dtype=np.int32))
        nd = np.ascontiguousarray(np.asarray(list(ndns), dtype=np.int32))
        h = _P()
        check("ed_opspace_create", lib().ed_opspace_create(self.norb, len(nu), nu.ctypes.data, len(nd),
                                                           nd.ctypes.data, ctypes.byref(h)))
        self._h = h
        a, b = _I64(), _I64()
        check("ed_opspace_dims", lib().ed_opspace_dims(h, ctypes.byref(a), ctypes.byref(b)))
        self.nsup, self.nsdn = a.value, b.value
        self.nstates = self.nsup * self.nsdn
        self._work = None

    def apply(self, terms, x, y=None, stream=None):
        """y = sum_t c_t (factors of t applied in list order) x.  terms:
        [(coeff, [(code, site1, spin1, site2, spin2), ...]), ...] as the
        reference's operator file encodes them; x, y device FP64 [nstates]."""
        import torch
        if x.dtype != torch.float64:
            raise TypeError("the operator engine works in FP64")
        if y is None:
            y = torch.empty(self.nstates, dtype=torch.float64, device=x.device)
        if self._work is None or self._work.device != x.device:
            self._work = torch.empty(2 * max(self.nstates, 1), dtype=torch.float64, device=x.device)
        off = np.zeros(len(terms) + 1, dtype=np.int32)
        flat, coeff = [], np.zeros(max(len(terms), 1), dtype=np.float64)
        for t, (c, ops) in enumerate(terms):
            coeff[t] = float(c)
            for o in ops:
                flat.append([int(v) for v in o])
            off[t + 1] = len(flat)
        ops_arr = np.ascontiguousarray(np.asarray(flat if flat else [[0] * 5], dtype=np.int32).reshape(-1, 5))
        wb = self._work.numel() * 8
        check("ed_ops_apply", lib().ed_ops_apply(self._h, _stream(stream), len(terms), off.ctypes.data,
                                                 ops_arr.ctypes.data, coeff.ctypes.data, _ptr(x, self.nstates, "x"),
                                                 _ptr(y, self.nstates, "y"), _ptr(self._work), int(wb)))
        return y

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ed_opspace_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """ed_batch: independent three-term Lanczos runs on their own sectors."""

    ROWS = (4, 8, 16)

    def __init__(self, sectors, rows: int = 8):
        self.sectors = list(sectors)
        arr = (_P * len(self.sectors))(*[s.handle.value for s in self.sectors])
        h = _P()
        check("ed_batch_create_rows", lib().ed_batch_create_rows(len(self.sectors), arr, int(rows), ctypes.byref(h)))
        self.rows = int(lib().ed_batch_rows(h))
        self._h = h
        tot, nb = _I64(), _I64()
        off = np.zeros(len(self.sectors), dtype=np.int64)
        sz = np.zeros(len(self.sectors), dtype=np.int64)
        check("ed_batch_layout", lib().ed_batch_layout(h, ctypes.byref(tot), off.ctypes.data, sz.ctypes.data,
                                                       ctypes.byref(nb)))
        self.total, self.offsets, self.sizes, self.nblocks = tot.value, off, sz, nb.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ed_batch_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view(self, vec, i):
        """Instance i's slot of a concatenated vector (internal layout of its sector)."""
        return vec[int(self.offsets[i]): int(self.offsets[i] + self.sizes[i])]

    def scratch_bytes(self):
        return int(lib().ed_batch_scratch_bytes(self._h))

    def hv(self, x, y, scratch, stream=None):
        """y_i = H_i x_i for every instance (concatenated batch layout)."""
        if y.dtype != x.dtype:
            raise TypeError("x and y must have the same dtype")
        check("ed_batch_hv", lib().ed_batch_hv(self._h, _stream(stream), dtype_code(x.dtype),
                                               _ptr(x, self.total, "x"), _ptr(y, self.total, "y"), _ptr(scratch),
                                               int(scratch.numel() * scratch.element_size())))

    def lanczos_persistent(self, work, x0, nsteps: int, alpha, beta, scratch, kept=None, stream=None):
        """The same run as lanczos() (kept=None; work 3*total) or lanczos_kept()
        (kept basis; work = y) in one persistent cooperative launch."""
        need = self.total if kept is not None else 3 * self.total
        if kept is not None:
            self._check(work, x0, nsteps, alpha, beta, work_need=self.total)
        else:
            self._check(work, x0, nsteps, alpha, beta)
        check("ed_batch_lanczos_persistent", lib().ed_batch_lanczos_persistent(
            self._h, _stream(stream), dtype_code(x0.dtype), _ptr(work, need, "work"), _ptr(x0, self.total, "x0"),
            int(nsteps), _ptr(alpha), _ptr(beta),
            None if kept is None else _ptr(kept, (int(nsteps) + 1) * self.total, "kept"), _ptr(scratch),
            int(scratch.numel() * scratch.element_size())))

    def persistent_status(self, scratch) -> int:
        st = _I()
        check("ed_batch_persistent_status", lib().ed_batch_persistent_status(self._h, _ptr(scratch),
                                                                             ctypes.byref(st)))
        return st.value

    def persistent_watchdog(self, wait_seconds: float = 10.0, stall_instance: int = -1):
        """Wait limit of later persistent runs, and (to test it) an instance
        whose first H*v phase never completes."""
        check("ed_batch_persistent_watchdog", lib().ed_batch_persistent_watchdog(self._h, float(wait_seconds),
                                                                                 int(stall_instance)))

    def lanczos(self, work, x0, nsteps: int, alpha, beta, scratch, stream=None):
        sb = scratch.numel() * scratch.element_size()
        self._check(work, x0, nsteps, alpha, beta)
        check("ed_batch_lanczos", lib().ed_batch_lanczos(self._h, _stream(stream), dtype_code(x0.dtype), _ptr(work),
                                                         _ptr(x0), int(nsteps), _ptr(alpha), _ptr(beta), _ptr(scratch),
                                                         int(sb)))

    def lanczos_kept(self, basis, y, x0, nsteps: int, alpha, beta, scratch, stream=None):
        """lanczos() keeping every Krylov vector: u_k in basis[k*total:(k+1)*total]."""
        sb = scratch.numel() * scratch.element_size()
        self._check(basis, x0, nsteps, alpha, beta, work_need=(int(nsteps) + 1) * self.total)
        if y.dtype != x0.dtype:
            raise TypeError("y and x0 must have the same dtype")
        tot = self.total
        check("ed_batch_lanczos_kept", lib().ed_batch_lanczos_kept(
            self._h, _stream(stream), dtype_code(x0.dtype), _ptr(basis, (int(nsteps) + 1) * tot, "basis"),
            _ptr(y, tot, "y"), _ptr(x0, tot, "x0"), int(nsteps), _ptr(alpha), _ptr(beta), _ptr(scratch), int(sb)))

    def ritz_sum(self, basis, nsteps: int, coef, beta, out, stream=None):
        """out_i = sum_k coef[i, k] u_k / beta[i, k] from a kept basis."""
        n, tot = len(self.sectors), self.total
        if out.dtype != basis.dtype:
            raise TypeError("out must have the dtype of the basis")
        check("ed_batch_ritz_sum", lib().ed_batch_ritz_sum(
            self._h, _stream(stream), dtype_code(basis.dtype), _ptr(basis, int(nsteps) * tot, "basis"), int(nsteps),
            _ptr(coef, n * int(nsteps), "coef"), _ptr(beta, n * (int(nsteps) + 1), "beta"), _ptr(out, tot, "out")))

    def ritz(self, work, x0, nsteps: int, alpha, beta, coef, out, scratch, stream=None):
        """Replay of lanczos() accumulating out_i += sum_k coef[i, k] q_k."""
        sb = scratch.numel() * scratch.element_size()
        self._check(work, x0, nsteps, alpha, beta)
        if out.dtype != x0.dtype:
            raise TypeError("out must have the dtype of x0")
        n = len(self.sectors)
        check("ed_batch_ritz", lib().ed_batch_ritz(self._h, _stream(stream), dtype_code(x0.dtype), _ptr(work),
                                                   _ptr(x0), int(nsteps), _ptr(alpha), _ptr(beta),
                                                   _ptr(coef, n * int(nsteps), "coef"), _ptr(out, self.total, "out"),
                                                   _ptr(scratch), int(sb)))

    def _check(self, work, x0, nsteps, alpha, beta, work_need=None):
        import torch
        n = len(self.sectors)
        if work.dtype != x0.dtype:
            raise TypeError("work and x0 must have the same dtype")
        if alpha.dtype != torch.float64 or beta.dtype != torch.float64:
            raise TypeError("alpha and beta are FP64")
        _ptr(work, 3 * self.total if work_need is None else work_need, "work")
        _ptr(x0, self.total, "x0")
        _ptr(alpha, n * int(nsteps), "alpha")
        _ptr(beta, n * (int(nsteps) + 1), "beta")


def gf_start(src: "Sector", dst: "Sector", kind: str, site: int, psi, out, stream=None):
    """out = c_{site}|psi> or c^+_{site}|psi> (kind 'h_up','h_down','e_up','e_down'),
    both vectors in their sectors' internal layouts."""
    check("ed_gf_start", lib().ed_gf_start(src.handle, dst.handle, _stream(stream), GF_KINDS[kind], int(site),
                                           dtype_code(psi.dtype), src.ld, _ptr(psi, src._need(src.ld), "psi"),
                                           dtype_code(out.dtype), dst.ld, _ptr(out, dst._need(dst.ld), "out")))


def gf_start_sites(src: "Sector", dst: "Sector", kind: str, sites, psi, out, stride: int, stream=None):
    """gf_start for several sites in one launch: site sites[j]'s vector starts
    j*stride elements into out (a 1-D tensor)."""
    sites = np.ascontiguousarray(np.asarray(sites, dtype=np.int32))
    ns = len(sites)
    need = (ns - 1) * int(stride) + dst._need(dst.ld) if ns else 0
    check("ed_gf_start_sites", lib().ed_gf_start_sites(
        src.handle, dst.handle, _stream(stream), GF_KINDS[kind], ns, sites.ctypes.data, dtype_code(psi.dtype), src.ld,
        _ptr(psi, src._need(src.ld), "psi"), dtype_code(out.dtype), dst.ld, _ptr(out, need, "out"), int(stride)))


def multidot(V, nvec: int, w, out, scratch, z=None, n: int | None = None, stream=None):
    """out[j] = <V_j, w> (and out[nvec+j] = <V_j, z>) for j < nvec, FP64 on device."""
    n = w.numel() if n is None else n
    ldv = V.stride(0) if V.dim() > 1 else n
    sb = scratch.numel() * scratch.element_size()
    check("ed_multidot", lib().ed_multidot(_stream(stream), dtype_code(V.dtype), int(n),
                                           _ptr(V, (int(nvec) - 1) * int(ldv) + int(n), "V"), int(ldv), int(nvec),
                                           _ptr(w, n, "w"), _ptr(z, n, "z"),
                                           _ptr(out, (2 if z is not None else 1) * int(nvec), "out"),
                                           _ptr(scratch), int(sb)))


def update(V, nvec: int, coef, w, out, norm2=None, scratch=None, n: int | None = None, stream=None, wscale=None):
    """out = ws w - sum_j coef_j V_j (w may be None), optional <out,out> into
    norm2; ws = wscale[0] (a device FP64 scalar, read on the device) or 1."""
    n = out.numel() if n is None else n
    ldv = V.stride(0) if (V is not None and V.dim() > 1) else n
    sb = 0 if scratch is None else scratch.numel() * scratch.element_size()
    vdt = dtype_code(V.dtype) if V is not None else dtype_code(out.dtype)
    needV = (int(nvec) - 1) * int(ldv) + int(n) if (V is not None and int(nvec) > 0) else None
    if wscale is not None:
        import torch
        if wscale.dtype != torch.float64:
            raise TypeError("wscale must be an FP64 device tensor")
    check("ed_update_wscaled", lib().ed_update_wscaled(
        _stream(stream), vdt, dtype_code(out.dtype), int(n), _ptr(V, needV, "V"), int(ldv), int(nvec),
        _ptr(coef, int(nvec), "coef"), _ptr(wscale, 1, "wscale"), _ptr(w, n, "w"), _ptr(out, n, "out"),
        _ptr(norm2, 1, "norm2"), _ptr(scratch), int(sb)))


def cf_eval(alpha, beta, z, shift=None, sign=None, stream=None):
    """Continued fractions of Lanczos coefficients (ed_cf_eval): [n, len(z)]
    complex128, instance i at z + shift[i] with sign[i] on H."""
    import torch
    n, m = int(alpha.shape[0]), int(alpha.shape[1])
    zc = z.to(torch.complex128).contiguous()
    out = torch.empty((n, zc.numel()), dtype=torch.complex128, device=alpha.device)
    a = alpha.to(torch.float64).contiguous()
    b = beta.to(torch.float64).contiguous()
    sh = None if shift is None else shift.to(torch.float64).contiguous()
    sg = None if sign is None else sign.to(torch.float64).contiguous()
    for i0 in range(0, n, 65535):
        i1 = min(n, i0 + 65535)
        check("ed_cf_eval", lib().ed_cf_eval(
            _stream(stream), i1 - i0, m, _ptr(a[i0:i1], (i1 - i0) * m, "alpha"),
            _ptr(b[i0:i1], (i1 - i0) * (m + 1), "beta"), zc.numel(), _ptr(torch.view_as_real(zc)),
            None if sh is None else _ptr(sh[i0:i1], i1 - i0, "shift"),
            None if sg is None else _ptr(sg[i0:i1], i1 - i0, "sign"), _ptr(torch.view_as_real(out[i0:i1]))))
    return out


def lanczos_state_doubles(mmax: int) -> int:
    """FP64 entries of the device state of ed_lanczos_coef for up to mmax steps."""
    v = int(lib().ed_lanczos_state_doubles(int(mmax)))
    if v < 0:
        raise ValueError(f"no Lanczos state for {mmax} steps (1..8192)")
    return v


def lanczos_coef(k: int, mmax: int, dots, nrm, state, coef, alpha, beta, stream=None):
    """Scalar work of step k of the full-reorthogonalisation Lanczos on the
    device (ed_lanczos_coef); dots=None only closes step k-1 (beta, scale)."""
    k, mmax = int(k), int(mmax)
    check("ed_lanczos_coef", lib().ed_lanczos_coef(
        _stream(stream), k, mmax, _ptr(dots, 2 * (k + 1), "dots"), _ptr(nrm, 1, "nrm"),
        _ptr(state, lanczos_state_doubles(mmax), "state"), _ptr(coef, k + 1, "coef"),
        _ptr(alpha, mmax, "alpha"), _ptr(beta, mmax, "beta")))
