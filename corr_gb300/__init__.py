"""corr_gb300: GB300-native correlation hot path of Masterluke87/corr.

The Python side of the C ABI (include/corr_gb300.h).  ``Context`` owns one
library context (device + stream + device workspace); array arguments may be
numpy arrays (host) or torch tensors (host or CUDA).  The functions below
mirror the reference's entry points (src/POSTHF/can_mp2.h, motrans.h, ri.h)
with explicit sizes instead of the reference's structs.
"""
from __future__ import annotations

import ctypes

from ._lib import (PRECISION, BasisC, CorrError, MP2Energy, RIMP2Instance, SystemInfo, Timing,
                   check, load)

__all__ = ["Basis", "Context", "CorrError", "MP2Energy", "PRECISION", "default_context",
           "read_system", "run_canonical_mp2_ri", "write_wav_hf"]


def _ptr(x):
    """Raw address of a numpy array or torch tensor (contiguous required)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr())
    if hasattr(x, "ctypes"):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return ctypes.c_void_p(x.ctypes.data)
    raise TypeError(f"unsupported array type {type(x)!r}")


def _prec(p):
    if isinstance(p, str):
        if p not in PRECISION:
            raise ValueError(f"unknown precision {p!r}; choose from {sorted(PRECISION)}")
        return PRECISION[p]
    return int(p)


class Basis:
    """Contracted Gaussian shells (corr_basis): l[s], nprim[s], poff[s],
    center[s][3] (bohr), exps and coefs of normalised primitives as in a
    basis-set file.  Functions: real solid harmonics m = -l..l per shell."""

    def __init__(self, l, nprim, poff, center, exps, coefs):
        import numpy as np

        self.l = np.ascontiguousarray(l, dtype=np.int32)
        self.nprim = np.ascontiguousarray(nprim, dtype=np.int32)
        self.poff = np.ascontiguousarray(poff, dtype=np.int32)
        self.center = np.ascontiguousarray(center, dtype=np.float64).reshape(-1)
        self.exps = np.ascontiguousarray(exps, dtype=np.float64)
        self.coefs = np.ascontiguousarray(coefs, dtype=np.float64)
        self.nbf = int(sum(2 * int(x) + 1 for x in self.l))

    def c(self):
        return BasisC(len(self.l), self.l.ctypes.data, self.nprim.ctypes.data,
                      self.poff.ctypes.data, self.center.ctypes.data, self.exps.ctypes.data,
                      self.coefs.ctypes.data)


class Context:
    """One corr_gb300 context on `device`, ordered on `stream` (a
    torch.cuda.Stream, a raw cudaStream_t integer, or None for the default
    stream)."""

    def __init__(self, device=0, stream=None):
        self._L = load()
        h = ctypes.c_void_p()
        check(self._L.corr_create(ctypes.byref(h), int(device), self._stream_ptr(stream)))
        self._h = h
        self.device = int(device)

    @staticmethod
    def _stream_ptr(stream):
        if stream is None:
            return None
        if hasattr(stream, "cuda_stream"):
            return ctypes.c_void_p(stream.cuda_stream)
        return ctypes.c_void_p(int(stream))

    def set_stream(self, stream):
        check(self._L.corr_set_stream(self._h, self._stream_ptr(stream)))

    @property
    def sm_count(self):
        return self._L.corr_device_sm_count(self._h)

    def set_timing(self, enable=True):
        check(self._L.corr_set_timing(self._h, 1 if enable else 0))

    def timing(self):
        """Device timings of the last call (needs set_timing(True))."""
        t = Timing()
        check(self._L.corr_get_timing(self._h, ctypes.byref(t)))
        return t

    def close(self):
        if getattr(self, "_h", None):
            self._L.corr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- RI-MP2 energy (src/POSTHF/can_mp2.cc:53) ---------------------------
    def rimp2_energy(self, bia, eps, nocc, nvir, naux, precision="fp64"):
        out = MP2Energy()
        check(self._L.corr_rimp2_energy(self._h, int(nocc), int(nvir), int(naux), _ptr(bia),
                                        _ptr(eps), _prec(precision), ctypes.byref(out)))
        return out

    def rimp2_energy_estimate(self, bia, eps, nocc, nvir, naux, precision="split_fp16"):
        """RI-MP2 energy and an estimate (one standard deviation) of its
        deviation from the FP64 energy of the same inputs.  Returns
        (MP2Energy, err)."""
        out = MP2Energy()
        err = ctypes.c_double(0.0)
        check(self._L.corr_rimp2_energy_estimate(self._h, int(nocc), int(nvir), int(naux),
                                                 _ptr(bia), _ptr(eps), _prec(precision),
                                                 ctypes.byref(out), ctypes.byref(err)))
        return out, err.value

    def rimp2_energy_async(self, bia, eps, nocc, nvir, naux, precision, out):
        """Enqueue only (device tensors; out = device float64[4] receiving
        E_SS, E_OS, E, E_SCS).  Capturable in a CUDA graph after a first call."""
        check(self._L.corr_rimp2_energy_async(self._h, int(nocc), int(nvir), int(naux),
                                              _ptr(bia), _ptr(eps), _prec(precision),
                                              _ptr(out)))

    def rimp2_gradient(self, bia, eps, nocc, nvir, naux, dbia=None, deps=None,
                       tensor_cores=False):
        """(E, dE/dB, dE/deps) of the RI-MP2 energy: FP64 (DMMA panels and the
        FP64 GEMM), or with tensor_cores the digit-GEMM form (FP64-accurate)."""
        dbia = self._out(bia, tuple(bia.shape), dbia)
        deps = self._out(eps, tuple(eps.shape), deps)
        e = MP2Energy()
        fn = self._L.corr_rimp2_gradient_tc if tensor_cores else self._L.corr_rimp2_gradient
        check(fn(self._h, int(nocc), int(nvir), int(naux), _ptr(bia), _ptr(eps), _ptr(dbia),
                 _ptr(deps), ctypes.byref(e)))
        return e.e_total, dbia, deps

    # -- batched RI-MP2 ---------------------------------------------------------
    @staticmethod
    def _instances(items):
        """items: iterable of (B[Q][i][a], eps, nocc, nvir) with device tensors."""
        items = list(items)
        arr = (RIMP2Instance * len(items))()
        for k, (B, e, o, v) in enumerate(items):
            arr[k].nocc, arr[k].nvir, arr[k].naux = int(o), int(v), int(B.shape[0])
            arr[k].bia = _ptr(B).value
            arr[k].eps = _ptr(e).value
        return arr, len(items)

    def rimp2_energy_batched(self, items, precision="split_bf16"):
        arr, n = self._instances(items)
        out = (MP2Energy * n)()
        check(self._L.corr_rimp2_energy_batched(self._h, n, arr, _prec(precision), out))
        return list(out)

    def rimp2_energy_batched_async(self, items, precision, out):
        """Enqueue only; out = device float64[4*n]. Capturable after a first call."""
        arr, n = self._instances(items)
        self._keep = arr  # the library copies the table during the call; keep for safety
        check(self._L.corr_rimp2_energy_batched_async(self._h, n, arr, _prec(precision),
                                                      _ptr(out)))

    def selftest_wait_timeout(self, limit_ms=50):
        """Run the kernels' bounded-wait path on purpose (raises CorrError with
        status CORR_ERR_DEVICE_TIMEOUT; the context stays usable)."""
        check(self._L.corr_selftest_wait_timeout(self._h, int(limit_ms)))

    def set_fp64_strict(self, strict=True):
        """Plain-form metric calls (ri_metric_inv_sqrt, calculate_ri) on the
        FP64 pipe only (True) or with the FP64-accurate digit GEMM (False,
        the default)."""
        check(self._L.corr_set_fp64_strict(self._h, 1 if strict else 0))

    def set_energy_tiles(self, tiles):
        """Accepts 0 or 1; no effect (every tile runs 128 wide)."""
        check(self._L.corr_set_energy_tiles(self._h, int(tiles)))

    def set_batch_policy(self, order, stages, tiles=1):
        check(self._L.corr_set_batch_policy(self._h, int(order), int(stages), int(tiles)))

    def batch_autotune(self, items, precision="split_bf16", cache=None):
        """Pick the batched launch variant (unit order, pipeline stages) by
        timing them on this batch.  With a cache path, results are
        stored per batch signature (sorted shape list) and reused without
        timing.  Returns (order, stages, tiles, ms)."""
        import hashlib
        import json
        import os

        items = list(items)
        sig = hashlib.sha1(json.dumps(sorted((int(B.shape[0]), int(o), int(v))
                                              for (B, _, o, v) in items)).encode()).hexdigest()
        key = f"{sig}:{precision}"
        db = {}
        if cache and os.path.exists(cache):
            try:
                with open(cache) as f:
                    db = json.load(f)
            except Exception:
                db = {}
        if key in db and "tiles" in db[key]:
            e = db[key]
            self.set_batch_policy(e["order"], e["stages"], e["tiles"])
            return e["order"], e["stages"], e["tiles"], e["ms"]
        arr, n = self._instances(items)
        order, stages, tiles, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        check(self._L.corr_rimp2_batch_autotune(self._h, n, arr, _prec(precision),
                                                ctypes.byref(order), ctypes.byref(stages),
                                                ctypes.byref(tiles), ctypes.byref(ms)))
        if cache:
            db[key] = {"order": order.value, "stages": stages.value, "tiles": tiles.value,
                       "ms": ms.value}
            d = os.path.dirname(os.path.abspath(cache))
            os.makedirs(d, exist_ok=True)
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(db, f, indent=1)
            os.replace(tmp, cache)
        return order.value, stages.value, tiles.value, ms.value

    def sync(self):
        check(self._L.corr_sync(self._h))

    # -- FP64 transforms (src/POSTHF/motrans.cc, ri.cc) and canonical MP2 ----
    @staticmethod
    def _out(like, shape, out):
        if out is not None:
            return out
        if hasattr(like, "device") and getattr(like, "is_cuda", False):
            import torch

            return torch.empty(shape, dtype=torch.float64, device=like.device)
        import numpy as np

        return np.zeros(shape)

    def build_fmo(self, mos, fmat, out=None):
        """build_FMo (motrans.cc:8): FMo = C F C^T with mos[p][mu]."""
        N = mos.shape[0]
        out = self._out(mos, (N, N), out)
        check(self._L.corr_build_fmo(self._h, N, _ptr(mos), _ptr(fmat), _ptr(out)))
        return out

    def motrans(self, nroe, mos, packed, out=None):
        """MOtrans (motrans.cc:35): full (ij|kl) from the packed AO list."""
        N = mos.shape[0]
        out = self._out(mos, (N, N, N, N), out)
        check(self._L.corr_motrans(self._h, nroe, N, _ptr(mos), packed.nrofint,
                                   _ptr(packed.sortcount), _ptr(packed.intval),
                                   _ptr(packed.intnums), _ptr(out)))
        return out

    def motrans_ovov(self, nroe, mos, packed, out=None):
        """(ia|jb) block [i][a][j][b] from the packed AO list."""
        N = mos.shape[0]
        o = nroe // 2
        v = N - o
        out = self._out(mos, (o, v, o, v), out)
        check(self._L.corr_motrans_ovov(self._h, nroe, N, _ptr(mos), packed.nrofint,
                                        _ptr(packed.sortcount), _ptr(packed.intval),
                                        _ptr(packed.intnums), _ptr(out)))
        return out

    def canonical_mp2(self, nroe, prec, eps):
        """run_canonical_mp2 (can_mp2.cc:11) on the full MO tensor."""
        out = MP2Energy()
        check(self._L.corr_canonical_mp2(self._h, nroe, prec.shape[0], _ptr(prec), _ptr(eps),
                                         ctypes.byref(out)))
        return out

    def canonical_mp2_ovov(self, ovov, eps):
        out = MP2Energy()
        o, v = ovov.shape[0], ovov.shape[1]
        check(self._L.corr_canonical_mp2_ovov(self._h, o, v, _ptr(ovov), _ptr(eps),
                                              ctypes.byref(out)))
        return out

    def transform_ri(self, nroe, mos, bpq, out=None):
        """transform_ri (ri.cc:147): Bia[Q][i][a] from BPQ[Q][mu][nu]."""
        X, N = bpq.shape[0], bpq.shape[1]
        o = nroe // 2
        out = self._out(bpq, (X, o, N - o), out)
        check(self._L.corr_transform_ri(self._h, nroe, N, X, _ptr(mos), _ptr(bpq), _ptr(out)))
        return out

    def ri_build_bpq(self, jm12, pmn, out=None):
        """BPQ = J^-1/2 (Q|mn) (ri.cc:102-103)."""
        X, N = pmn.shape[0], pmn.shape[1]
        out = self._out(pmn, (X, N, N), out)
        check(self._L.corr_ri_build_bpq(self._h, X, N, _ptr(jm12), _ptr(pmn), _ptr(out)))
        return out

    def ri_metric_inv_sqrt(self, J, tol=1e-10, out=None):
        """J^-1/2 with the reference's eigenvalue cutoff (ri.cc:50-69).
        Returns (jm12, ncut)."""
        X = J.shape[0]
        out = self._out(J, (X, X), out)
        ncut = ctypes.c_int(0)
        check(self._L.corr_ri_metric_inv_sqrt(self._h, X, _ptr(J), float(tol), _ptr(out),
                                              ctypes.byref(ncut)))
        return out, ncut.value

    def calculate_ri(self, J, pmn, out=None):
        """calculate_ri (ri.cc:7) downstream of the integrals: BPQ = J^-1/2 (Q|mn)."""
        X, N = pmn.shape[0], pmn.shape[1]
        out = self._out(pmn, (X, N, N), out)
        check(self._L.corr_calculate_ri(self._h, X, N, _ptr(J), _ptr(pmn), _ptr(out)))
        return out

    def ri_apply_metric(self, jm12, x, out=None):
        """out = jm12 @ x for x [naux][...] (the metric applied to (P|ia))."""
        X = jm12.shape[0]
        ncols = int(x.size // X) if hasattr(x, "size") and not callable(x.size) else int(x.numel() // X)
        out = self._out(x, tuple(x.shape), out)
        check(self._L.corr_ri_apply_metric(self._h, X, ncols, _ptr(jm12), _ptr(x), _ptr(out)))
        return out

    def rimp2_energy_from_3index(self, nroe, mos, eps, J, pmn, precision="split_bf16"):
        """RI-MP2 energy from (P|mu nu), J, MO coefficients mos[p][mu] and
        orbital energies, entirely on the GPU.  Returns (MP2Energy, ncut)."""
        X, N = pmn.shape[0], pmn.shape[1]
        out = MP2Energy()
        ncut = ctypes.c_int(0)
        check(self._L.corr_rimp2_energy_from_3index(self._h, int(nroe), N, X, _ptr(mos), _ptr(eps),
                                                    _ptr(J), _ptr(pmn), _prec(precision),
                                                    ctypes.byref(out), ctypes.byref(ncut)))
        return out, ncut.value

    # -- RI integrals (the libint part of calculate_ri, src/POSTHF/ri.cc) -----
    def ri_integrals(self, obs, aux, device="cuda", metric=True, three_index=True):
        """(J[X][X], pmn[X][N][N]) = ((P|Q), (P|mu nu)) for Basis objects obs
        and aux, computed on the GPU; outputs as CUDA tensors (device="cuda")
        or numpy arrays."""
        X = aux.nbf
        J = self._filled(device, (X, X), "float64", None) if metric else None
        P = (self._filled(device, (X, obs.nbf, obs.nbf), "float64", None)
             if three_index else None)
        bo, ba = obs.c() if obs is not None else None, aux.c()
        check(self._L.corr_ri_integrals(self._h, ctypes.byref(bo) if bo is not None else None,
                                        ctypes.byref(ba), _ptr(J), _ptr(P)))
        return J, P

    # -- CCSD consumer of the MO integrals (src/POSTHF/ccsd.cc) --------------
    def ints_so(self, prec, out=None):
        """calc_ints_so (ccsd.cc:509): <ij||kl> over 2N spin orbitals from the
        spatial MO integrals prec[N][N][N][N] (corr_motrans layout)."""
        N = prec.shape[0]
        out = self._out(prec, (2 * N,) * 4, out)
        check(self._L.corr_ints_so(self._h, N, _ptr(prec), _ptr(out)))
        return out

    def cc_fock(self, nroe, mos, hmat, prec):
        """form_fock (ccsd.cc:11): spin-orbital (h, f), each 2N x 2N."""
        N = mos.shape[0]
        h = self._out(prec, (2 * N, 2 * N), None)
        f = self._out(prec, (2 * N, 2 * N), None)
        check(self._L.corr_cc_fock(self._h, int(nroe), N, _ptr(mos), _ptr(hmat), _ptr(prec),
                                   _ptr(h), _ptr(f)))
        return h, f

    # -- RHF (src/SCF) --------------------------------------------------------
    def build_fmat(self, pmat, hmat, sortcount, intval, intnums, out=None):
        """build_Fmat (ops_rhf.cc:549): F = H + sum P ((mn|ls) - 1/2 (ml|ns))."""
        N = pmat.shape[0]
        out = self._out(pmat, (N, N), out)
        check(self._L.corr_build_fmat(self._h, N, _ptr(pmat), _ptr(hmat), int(intval.shape[0]),
                                      _ptr(sortcount), _ptr(intval), _ptr(intnums), _ptr(out)))
        return out

    def run_scf(self, nroe, smat, hmat, sortcount, intval, intnums, mos=None, ion_rep=0.0,
                maxiter=100):
        """run_scf (scf.cc:145): RHF on the GPU.  ``mos`` (orbitals as rows)
        is the guess; None or a near-zero diagonal takes the core guess.
        Returns a dict with mos, fmat, moens, the energies run_scf prints
        (total, one, two) and the iteration count."""
        import numpy as np

        N = smat.shape[0]
        on_dev = hasattr(smat, "is_cuda") and smat.is_cuda
        if mos is None:
            mos = self._out(smat, (N, N), None)
            mos[...] = 0
        else:
            mos = mos.clone() if on_dev else np.array(mos, dtype=np.float64, copy=True)
        fmat = self._out(smat, (N, N), None)
        pmat = self._out(smat, (N, N), None)
        moens = self._out(smat, (N,), None)
        e = np.zeros(3)
        it = ctypes.c_int(0)
        check(self._L.corr_run_scf(self._h, int(nroe), N, float(ion_rep), _ptr(smat), _ptr(hmat),
                                   int(intval.shape[0]), _ptr(sortcount), _ptr(intval),
                                   _ptr(intnums), int(maxiter), _ptr(mos), _ptr(fmat),
                                   _ptr(moens), _ptr(e), ctypes.byref(it), _ptr(pmat)))
        return {"mos": mos, "fmat": fmat, "pmat": pmat, "moens": moens, "energy": float(e[0]),
                "one": float(e[1]), "two": float(e[2]), "iterations": it.value}

    # -- hand-off files (src/IO/ops_io.cc) -----------------------------------
    # Output arrays may be numpy arrays or torch tensors (CUDA tensors are
    # filled through pinned chunk buffers on the context stream).
    def _filled(self, like, shape, dtype, out):
        if out is not None:
            return out
        import numpy as np

        dtype = np.dtype(dtype).type
        if like == "cuda":
            import torch

            return torch.empty(shape, dtype={np.float64: torch.float64, np.int64: torch.int64,
                                             np.uint16: torch.int16}[dtype],
                               device=f"cuda:{self.device}")
        return np.empty(shape, dtype=dtype)

    def read_oei(self, prefix, nroao, device="cpu"):
        """read_oei (ops_io.cc:112): (H, T, S, V) of PREFIX.oei."""
        import numpy as np

        mats = [self._filled(device, (nroao, nroao), np.float64, None) for _ in range(4)]
        check(self._L.corr_read_oei(self._h, prefix.encode(), int(nroao), *[_ptr(m) for m in mats]))
        return tuple(mats)

    def read_tei(self, prefix, nrofint, device="cpu"):
        """read_tei (ops_io.cc:203): (sortcount[4], intval, intnums[nrofint][4])."""
        import numpy as np

        sc = np.zeros(4, dtype=np.int64)
        iv = self._filled(device, (int(nrofint),), np.float64, None)
        inum = self._filled(device, (int(nrofint), 4), np.uint16, None)
        check(self._L.corr_read_tei(self._h, prefix.encode(), int(nrofint), _ptr(sc), _ptr(iv),
                                    _ptr(inum)))
        return sc, iv, inum

    def read_wav_hf(self, prefix, nroao, device="cpu"):
        """read_wav_HF (ops_io.cc:283): (MO energies, MO coefficients [p][mu])."""
        import numpy as np

        e = self._filled(device, (nroao,), np.float64, None)
        c = self._filled(device, (nroao, nroao), np.float64, None)
        check(self._L.corr_read_wav_hf(self._h, prefix.encode(), int(nroao), _ptr(e), _ptr(c)))
        return e, c

    def read_rimp2(self, prefix, naux, nroao, device="cpu"):
        """BPQ[naux][nroao][nroao] of PREFIX.rimp2 (read by read_transform_ri, ri.cc:109)."""
        import numpy as np

        b = self._filled(device, (naux, nroao, nroao), np.float64, None)
        check(self._L.corr_read_rimp2(self._h, prefix.encode(), int(naux), int(nroao), _ptr(b)))
        return b

    # -- dense FP64 helpers (src/MATH/ops_mat.cc) ----------------------------
    def dgemm(self, A, B, transa=False, transb=False, alpha=1.0, beta=0.0, out=None,
              tensor_cores=False):
        """C = alpha op(A) op(B) + beta C for row-major 2-D arrays (mat_mat_T:
        transb, mat_T_mat: transa).  `out` is read when beta != 0.
        tensor_cores: the FP64-accurate digit-sliced form (corr_dgemm_tc)."""
        m = A.shape[1] if transa else A.shape[0]
        k = A.shape[0] if transa else A.shape[1]
        n = B.shape[0] if transb else B.shape[1]
        if (B.shape[1] if transb else B.shape[0]) != k:
            raise ValueError("dgemm: inner dimensions differ")
        if beta != 0.0 and out is None:
            raise ValueError("dgemm: beta != 0 needs out")
        out = self._out(A, (m, n), out)
        fn = self._L.corr_dgemm_tc if tensor_cores else self._L.corr_dgemm
        check(fn(self._h, int(transa), int(transb), m, n, k, float(alpha), _ptr(A), A.shape[1],
                 _ptr(B), B.shape[1], float(beta), _ptr(out), n))
        return out

    def syev(self, A, w=None, vecs=None):
        """diag_mat (ops_mat.cc:21): eigenvalues ascending and vecs[k] =
        eigenvector k of the symmetric matrix A (its row-major lower triangle
        is read, as dsyev reads it there)."""
        n = A.shape[0]
        w = self._out(A, (n,), w)
        vecs = self._out(A, (n, n), vecs)
        check(self._L.corr_syev(self._h, n, _ptr(A), _ptr(w), _ptr(vecs)))
        return w, vecs


def read_system(prefix):
    """read_system (ops_io.cc:63): (SystemInfo, coord[nroa][3], charges, zeff,
    mass) of PREFIX.sys.  Host arrays; needs no GPU."""
    import numpy as np

    L = load()
    info = SystemInfo()
    check(L.corr_read_system(prefix.encode(), ctypes.byref(info), None, None, None, None))
    na = info.nroa
    coord = np.empty((na, 3))
    charges, zeff, mass = np.empty(na), np.empty(na), np.empty(na)
    check(L.corr_read_system(prefix.encode(), ctypes.byref(info), _ptr(coord), _ptr(charges),
                             _ptr(zeff), _ptr(mass)))
    return info, coord, charges, zeff, mass


def write_wav_hf(path, moens, mos):
    """write_wav_HF (ops_io.cc:259) of host arrays."""
    check(load().corr_write_wav_hf(path.encode(), int(moens.shape[0]), _ptr(moens), _ptr(mos)))


def read_files_host(prefix, nroao, nrofint):
    """The packed ERIs and one-electron matrices of PREFIX.tei/.oei into host
    arrays without a context or GPU (the readers' host path)."""
    import numpy as np

    L = load()
    mats = [np.empty((nroao, nroao)) for _ in range(4)]
    check(L.corr_read_oei(None, prefix.encode(), int(nroao), *[_ptr(m) for m in mats]))
    sc = np.zeros(4, dtype=np.int64)
    iv = np.empty(int(nrofint))
    inum = np.empty((int(nrofint), 4), dtype=np.uint16)
    check(L.corr_read_tei(None, prefix.encode(), int(nrofint), _ptr(sc), _ptr(iv), _ptr(inum)))
    return tuple(mats), (sc, iv, inum)


_DEFAULT = None


def default_context():
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


def run_canonical_mp2_ri(nroe, nroao, naux_2, Bia, FMo_diag, precision="fp64", ctx=None):
    """Mirror of run_canonical_mp2_ri(systeminfo*, pHF*) (can_mp2.cc:53):
    nroe electrons, nroao orbitals, naux_2 auxiliary functions, Bia[Q][i][a],
    FMo_diag[nroao] = orbital energies.  Returns MP2Energy."""
    nocc = nroe // 2
    return (ctx or default_context()).rimp2_energy(Bia, FMo_diag, nocc, nroao - nocc, naux_2,
                                                   precision)
