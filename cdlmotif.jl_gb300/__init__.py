"""cdlgb -- GB300-native convolutional-dictionary-learning hot path of CDLmotif.jl.

Host-side mirror of the reference's Julia interface for the hot path.  Every
compute call goes through the C ABI of ``libcdlgb.so`` (include/cdlgb.h); there is
no CPU fallback.  Names follow the reference (a trailing ``!`` becomes nothing):

=====================  =========================================================
this module            reference (kchu25/CDLmotif.jl)
=====================  =========================================================
CDLSetup               CDL_setup          src/SETUP/WRAPPER_setup.jl:1-13
init_cdl -> CDL        init_cdl / cdl     src/SETUP/CDL_setup.jl:165-283
code_update            code_update!       src/CDL/train.jl:1-44
dict_update            dict_update!       src/CDL/train.jl:46-89
update_best            update_best!       src/CDL/train.jl:91-98
objective              objective          src/SETUP/CDL_setup.jl:286
cdl_train              one training of cdl_optimize   src/WRAPPER/wrap.jl:5-12
scan_w_gpu             scan_w_gpu!        src/SEARCH/scan.jl:176-221
overlapping_scan       overlapping_scan!  src/SEARCH/scan.jl:89-121
posdicts2pfms          posdicts2pfms      src/SEARCH/helpers.jl:59-96
pfm2pwm                pfm2pwm            src/SEARCH/helpers.jl:12-13
save_pfms_as_transfac  save_pfms_as_transfac  src/SAVE/save_learned_results.jl:184-217
=====================  =========================================================

Array layouts: a Julia column-major array of dims (a, b, c) is a C-order numpy
array of shape (c, b, a) -- e.g. the one-hot data (4L, N) is numpy (N, 4L), X is
numpy (N, M, Lg), D is numpy (M, Lg), pwms (K, 4, maxlen) is numpy (maxlen, 4, K).

Errors raise ``CDLGBError`` (never ValueError/ArgumentError-like types: the
reference's retry loop, src/WRAPPER/wrap.jl:141, treats ArgumentError as "no motif
found, relax and retry").
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import synth
from ._lib import CdlgbParams, ptr

__all__ = ["CDLSetup", "CDL", "CDLGBError", "init_cdl", "code_update", "dict_update",
           "update_best", "objective", "cdl_train", "scan_w_gpu", "overlapping_scan",
           "posdicts2pfms", "count_matrices", "pfm2pwm", "pwm_complement",
           "save_pfms_as_transfac", "transfac_text", "FIELDS", "build", "ActivationRecord",
           "non_overlap_scan", "get_thresh", "extension", "extend", "trim_pfms", "masked_trim",
           "scores_reevaluation", "fisher_evalues", "filter_using_evalue",
           "record_training_result", "get_spatial_info", "get_pair_pfms", "select_pairs"]

FIELDS = {"X": 0, "X_best": 1, "d": 2, "D_best": 3, "G1": 4, "G3": 5, "DX": 6, "Y1": 7,
          "y2": 8, "y3": 9, "g1": 10, "g3": 11, "Td": 12, "G2": 13, "g2": 14, "y1": 15}
_LMN = {"X", "X_best", "d", "y2", "y3", "g1", "g3"}
_LN = {"DX", "Y1", "Td", "G2", "g2", "y1"}
_LM = {"D_best", "G1", "G3"}


class CDLGBError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"cdlgb {_lib.STATUS.get(status, status)}: {msg}")
        self.status = status


def build(verbose: bool = False) -> str:
    from . import buildlib as _b
    return _b.build(verbose=verbose)


@dataclass
class CDLSetup:
    """CDL_setup (src/SETUP/WRAPPER_setup.jl:1-13), same defaults."""
    M: int = 10
    filter_size: int = 4
    rho: float = 100.0
    sigma: float = 100.0
    lambda_: float = 0.01
    count_threshold: int = 50
    csc_iter_num: int = 15
    cdl_iter_num: int = 1
    iter_num: int = 10
    std_threshold_multiplier: float = 1.0
    num_train: int = 2
    stop_tol: float = 0.0     # stopping test of run_outer; 0 = the reference's fixed count
    track_residuals: bool = False   # keep the FP64 residual record (implied by stop_tol > 0)

    def params(self, device: int = 0, fft_mode: int = 0, init_mode: int = 0,
               hbm_budget_bytes: int = 0) -> CdlgbParams:
        p = CdlgbParams()
        _lib.lib().cdlgb_params_default(C.byref(p))
        p.M, p.filter_size = int(self.M), int(self.filter_size)
        p.rho, p.sigma, p.lambda_ = float(self.rho), float(self.sigma), float(self.lambda_)
        p.csc_iter_num, p.cdl_iter_num = int(self.csc_iter_num), int(self.cdl_iter_num)
        p.iter_num = int(self.iter_num)
        p.std_threshold_multiplier = float(self.std_threshold_multiplier)
        p.device, p.fft_mode, p.init_mode = int(device), int(fft_mode), int(init_mode)
        p.hbm_budget_bytes = int(hbm_budget_bytes)
        p.stop_tol = float(self.stop_tol)
        p.track_residuals = 1 if self.track_residuals else 0
        return p


def _check(ctx, st: int):
    if st != 0:
        msg = _lib.lib().cdlgb_last_error(ctx)
        raise CDLGBError(st, msg.decode() if msg else "")


class CDL:
    """Handle to one dataset's ADMM state resident on the GPU (the reference's
    ``cdl`` struct, src/SETUP/CDL_setup.jl:70-163).  Fields are downloaded on
    access; ``L`` is 4 x bases as in the reference."""

    def __init__(self, setup: CDLSetup, device: int = 0, fft_mode: int = 0,
                 init_mode: int = 0, hbm_budget_bytes: int = 0):
        L = _lib.lib()
        self.setup = setup
        self._p = setup.params(device, fft_mode, init_mode, hbm_budget_bytes)
        h = C.c_void_p()
        st = L.cdlgb_create(C.byref(self._p), C.byref(h))
        if st != 0:
            raise CDLGBError(st, L.cdlgb_last_error(None).decode())
        self._h = h
        self.N = self.M = self.L = self.gamma = self.Lg = None

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().cdlgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- data
    def load_data(self, data_matrix: np.ndarray):
        S = np.ascontiguousarray(data_matrix, dtype=np.float32)
        if S.ndim != 2:
            raise CDLGBError(-1, "data_matrix must be (N, 4L)")
        N, L4 = S.shape
        _check(self._h, _lib.lib().cdlgb_load_data(self._h, ptr(S, C.c_float), L4, N))
        d = [C.c_int32() for _ in range(5)]
        _check(self._h, _lib.lib().cdlgb_dims(self._h, *[C.byref(x) for x in d]))
        self.L, self.N, self.M, self.gamma, self.Lg = [x.value for x in d]

    def load_fasta(self, fasta, max_entries: int = 10000) -> dict:
        """read_fasta + data_2_dummy (src/LOAD/read.jl:2-28, src/LOAD/to_dummy.jl:27-38):
        `fasta` is FASTA text (str or bytes) or a path; records with 'N'/'n' are dropped,
        the first `max_entries` kept and one-hot encoded on the GPU.  Returns
        {"N", "L", "wrong_length"} (records whose length differs from the first one's
        are zero columns)."""
        if isinstance(fasta, (str, os.PathLike)) and os.path.exists(fasta):
            with open(fasta, "rb") as f:
                text = f.read()
        else:
            text = fasta.encode() if isinstance(fasta, str) else bytes(fasta)
        n, l, w = C.c_int32(), C.c_int32(), C.c_int32()
        _check(self._h, _lib.lib().cdlgb_load_fasta(self._h, text, len(text), int(max_entries),
                                                    C.byref(n), C.byref(l), C.byref(w)))
        d = [C.c_int32() for _ in range(5)]
        _check(self._h, _lib.lib().cdlgb_dims(self._h, *[C.byref(x) for x in d]))
        self.L, self.N, self.M, self.gamma, self.Lg = [x.value for x in d]
        return {"N": n.value, "L": l.value, "wrong_length": w.value}

    def data(self) -> np.ndarray:
        """The loaded one-hot data, (N, 4L) float32 (== Julia (4L, N))."""
        out = np.empty((self.N, self.L), np.float32)
        _check(self._h, _lib.lib().cdlgb_get(self._h, 17, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def make_background(self, k: int = 3, seed: int = 0):
        """The background of the e-value filter on the device: every sequence k-let
        shuffled (the reference runs `fasta-shuffle-letters -kmer 3`,
        src/SETUP/LOAD_setup.jl:8)."""
        _check(self._h, _lib.lib().cdlgb_make_background(self._h, int(k), int(seed) & (2**64 - 1)))

    def background(self) -> np.ndarray:
        """The background one-hot matrix (N, 4L) float32."""
        out = np.empty((self.N, self.L), np.float32)      # self.L holds 4L
        _check(self._h, _lib.lib().cdlgb_get(self._h, 18, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def select_data(self, which: int):
        """0: scans / counts / refinement read the data; 1: they read the background."""
        _check(self._h, _lib.lib().cdlgb_select_data(self._h, int(which)))

    def on_background(self):
        """Context manager: the scan family reads the background inside the block."""
        import contextlib

        @contextlib.contextmanager
        def cm():
            self.select_data(1)
            try:
                yield self
            finally:
                self.select_data(0)
        return cm()

    def autotune(self) -> dict:
        """Time every fused X-step variant for this dataset's shape on a prefix of the
        sequences and keep the fastest (cdlgb_autotune).  Returns the candidates with
        their ms per X-step and the chosen index."""
        maxc = 16
        ms = np.zeros(maxc, np.float64)
        kind, cs, mc = (np.zeros(maxc, np.int32) for _ in range(3))
        n, ch = C.c_int32(), C.c_int32()
        _check(self._h, _lib.lib().cdlgb_autotune(self._h, maxc, ms.ctypes.data_as(C.POINTER(C.c_double)),
                                                  ptr(kind, C.c_int32), ptr(cs, C.c_int32), ptr(mc, C.c_int32),
                                                  C.byref(n), C.byref(ch)))
        k = n.value
        names = {1: "multi-iteration", 2: "one-X-step"}
        cands = [{"kernel": names[int(kind[i])], "cluster": int(cs[i]), "filters_per_cta": int(mc[i]),
                  "ms_per_xstep": float(ms[i])} for i in range(k)]
        return {"candidates": cands, "chosen": ch.value}

    def init_state(self, X0=None, D0=None, seed: int = 0):
        X0c = None if X0 is None else np.ascontiguousarray(X0, np.float32).reshape(self.N, self.M, self.Lg)
        D0c = None if D0 is None else np.ascontiguousarray(D0, np.float32).reshape(self.M, self.Lg)
        _check(self._h, _lib.lib().cdlgb_init_state(self._h, ptr(X0c, C.c_float),
                                                    ptr(D0c, C.c_float), C.c_uint64(seed)))

    # -- fields
    def get(self, name: str) -> np.ndarray:
        if name == "obj_best":
            return self.obj_best
        if name in _LMN:
            shape = (self.N, self.M, self.Lg)
        elif name in _LN:
            shape = (self.N, self.Lg)
        elif name in _LM:
            shape = (self.M, self.Lg)
        else:
            raise CDLGBError(-1, f"unknown field {name}")
        out = np.empty(shape, np.float32)
        _check(self._h, _lib.lib().cdlgb_get(self._h, FIELDS[name], out.ctypes.data_as(C.c_void_p),
                                             out.nbytes))
        return out

    RESIDUALS = ("x_y2", "x_y3", "x_y1", "x_norm", "dx_norm", "d_g1", "d_g3", "d_g2", "d_norm",
                 "td_norm", "dual_G1", "dual_G3", "G_norm", "rel_primal_x", "rel_primal_dx",
                 "rel_primal_d", "rel_primal_td", "rel_dual_d", "rel_max")

    def residuals(self) -> np.ndarray:
        """The residual record (19 float64, include/cdlgb.h: primal residuals of the last
        code update's final iterate, the last D-step's dual increments and consensus
        change, the relative residuals of the stopping test)."""
        out = np.zeros(19, np.float64)
        _check(self._h, _lib.lib().cdlgb_get(self._h, 19, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def relative_residuals(self) -> dict:
        return dict(zip(self.RESIDUALS[13:], (float(v) for v in self.residuals()[13:])))

    @property
    def outer_done(self) -> int:
        v = C.c_int32()
        _check(self._h, _lib.lib().cdlgb_get(self._h, 20, C.cast(C.byref(v), C.c_void_p), 4))
        return v.value

    @property
    def obj_best(self) -> float:
        v = C.c_double()
        _check(self._h, _lib.lib().cdlgb_get(self._h, 16, C.cast(C.byref(v), C.c_void_p), 8))
        return v.value

    def __getattr__(self, name):
        if name in FIELDS:
            return self.get(name)
        raise AttributeError(name)

    # -- instrumentation
    def set_stream(self, stream_ptr: int | None):
        _check(self._h, _lib.lib().cdlgb_set_stream(self._h, C.c_void_p(stream_ptr or 0) if stream_ptr else None))

    def profile(self, enable: bool = True):
        _check(self._h, _lib.lib().cdlgb_profile(self._h, 1 if enable else 0))

    PHASES = ("xstep", "dstep", "objective", "xfused", "setup", "threshold", "scan", "spare")

    def profile_read(self, reset: bool = True) -> dict:
        ms = (C.c_double * 8)()
        cnt = (C.c_int64 * 8)()
        la, ff = C.c_int64(), C.c_int64()
        _check(self._h, _lib.lib().cdlgb_profile_read(self._h, ms, cnt, C.byref(la), C.byref(ff),
                                                      1 if reset else 0))
        out = {p: (ms[i], cnt[i]) for i, p in enumerate(self.PHASES)}
        out["launches"] = la.value
        out["fft_calls"] = ff.value
        return out


# ---------------------------------------------------------------------------- ADMM
def init_cdl(cdl_setup: CDLSetup, data_matrix: np.ndarray, X0=None, D0=None, seed: int = 0,
             device: int = 0, fft_mode: int = 0, init_mode: int = 0,
             hbm_budget_bytes: int = 0) -> CDL:
    """init_cdl (src/SETUP/CDL_setup.jl:273-283): upload the one-hot data (N, 4L),
    allocate the state and initialise it.  X0 (N, M, Lg) / D0 (M, Lg) replace the
    reference's unseeded random draws when given."""
    c = CDL(cdl_setup, device=device, fft_mode=fft_mode, init_mode=init_mode,
            hbm_budget_bytes=hbm_budget_bytes)
    c.load_data(data_matrix)
    c.init_state(X0, D0, seed)
    return c


def code_update(c: CDL, num_iter: int):
    """code_update! (src/CDL/train.jl:1-44)."""
    _check(c._h, _lib.lib().cdlgb_code_update(c._h, int(num_iter)))


def dict_update(c: CDL, num_iter: int):
    """dict_update! (src/CDL/train.jl:46-89)."""
    _check(c._h, _lib.lib().cdlgb_dict_update(c._h, int(num_iter)))


def objective(c: CDL) -> float:
    """objective (src/SETUP/CDL_setup.jl:286), float64."""
    v = C.c_double()
    _check(c._h, _lib.lib().cdlgb_objective(c._h, C.byref(v)))
    return v.value


def update_best(c: CDL) -> tuple[float, bool]:
    """update_best! (src/CDL/train.jl:91-98).  Returns (objective, improved)."""
    v, imp = C.c_double(), C.c_int32()
    _check(c._h, _lib.lib().cdlgb_update_best(c._h, C.byref(v), C.byref(imp)))
    return v.value, bool(imp.value)


def run_outer(c: CDL, iter_num: int) -> np.ndarray:
    """iter_num passes of cdl_optimize's loop body (src/WRAPPER/wrap.jl:6-11); fewer
    when the setup's stop_tol > 0 and the stopping test passes (one objective per pass
    run)."""
    objs = np.zeros(max(iter_num, 1), np.float64)
    _check(c._h, _lib.lib().cdlgb_run_outer(c._h, int(iter_num), ptr(objs, C.c_double)))
    return objs[:c.outer_done]


def code_threshold(c: CDL) -> float:
    """std_threshold_multiplier * std(X_best[X_best .> 0]) (src/WRAPPER/wrap.jl:12)."""
    v = C.c_double()
    _check(c._h, _lib.lib().cdlgb_code_threshold(c._h, C.byref(v)))
    return v.value


def cdl_train(cdl_setup: CDLSetup, data_matrix: np.ndarray, X0=None, D0=None, seed: int = 0,
              verbose: bool = False, **kw):
    """One training of cdl_optimize (src/WRAPPER/wrap.jl:5-12): init, iter_num outer
    iterations, code threshold.  Returns (CDL handle, code_thresh, objectives)."""
    c = init_cdl(cdl_setup, data_matrix, X0, D0, seed, **kw)
    objs = []
    for it in range(1, cdl_setup.iter_num + 1):
        code_update(c, cdl_setup.csc_iter_num)
        o, _ = update_best(c)
        dict_update(c, cdl_setup.cdl_iter_num)
        objs.append(o)
        if verbose and it % 5 == 0:
            print("obj: ", round(objective(c), 2))
    return c, code_threshold(c), objs


# ---------------------------------------------------------------------------- search
def _pack_pwms(pwms, lens=None):
    """List of (4, w_k) PWMs -> (maxlen, 4, K) float32 (Julia (K, 4, maxlen)), zero padded."""
    K = len(pwms)
    if lens is None:
        lens = [np.asarray(p).shape[1] for p in pwms]
    lens = np.asarray(lens, np.int32)
    maxlen = int(lens.max())
    arr = np.zeros((maxlen, 4, K), np.float32)
    for k, p in enumerate(pwms):
        p = np.asarray(p, np.float32)
        arr[: lens[k], :, k] = p[:, : lens[k]].T
    return np.ascontiguousarray(arr), lens, maxlen


def scan_w_gpu(c: CDL, pwms, thresh, lens=None) -> np.ndarray:
    """scan_w_gpu! + greedy_search! (src/SEARCH/scan.jl:176-239) on c's data.
    Returns positions int32 (N, K) == Julia (K, N): 1-based argmax of the
    thresholded forward-strand score, 0 = not found (position 1 also reads 0)."""
    arr, lens, maxlen = _pack_pwms(pwms, lens)
    K = len(lens)
    th = np.ascontiguousarray(thresh, np.float32)
    out = np.zeros((c.N, K), np.int32)
    _check(c._h, _lib.lib().cdlgb_scan_fwd(c._h, ptr(arr, C.c_float), ptr(lens, C.c_int32),
                                           ptr(th, C.c_float), K, maxlen, ptr(out, C.c_int32)))
    return out


def positions_to_dicts(pos: np.ndarray) -> list[dict]:
    """(N, K) positions -> one Dict(n => pos) per motif, 1-based n, as scan_w_gpu!
    builds them (scan.jl:200-205)."""
    N, K = pos.shape
    return [{int(n) + 1: int(pos[n, k]) for n in np.nonzero(pos[:, k])[0]} for k in range(K)]


def overlapping_scan(c: CDL, pwms, thresh, lens=None):
    """overlapping_scan! (src/SEARCH/scan.jl:89-121): both strands.  Returns
    (positions int32 (N, K), scores float32 (N, K), use_comp uint8 (N, K)); position
    0 = no score above the threshold."""
    arr, lens, maxlen = _pack_pwms(pwms, lens)
    K = len(lens)
    th = np.ascontiguousarray(thresh, np.float32)
    pos = np.zeros((c.N, K), np.int32)
    sc = np.zeros((c.N, K), np.float32)
    uc = np.zeros((c.N, K), np.uint8)
    _check(c._h, _lib.lib().cdlgb_scan_both(c._h, ptr(arr, C.c_float), ptr(lens, C.c_int32),
                                            ptr(th, C.c_float), K, maxlen, ptr(pos, C.c_int32),
                                            ptr(sc, C.c_float), ptr(uc, C.c_uint8)))
    return pos, sc, uc


def get_thresh(c: CDL, pwms, pval: float = 2.7e-4, lens=None) -> np.ndarray:
    """get_thresh (src/SEARCH/helpers.jl:99): Float32(pvalue2score(pwm, pval)) per PWM
    (Touzet-Varre score distribution, src/SEARCH/PWM_Touzet.jl:199-217), batched on
    the GPU with exact integer counts.  Returns float32 (K,)."""
    arr, lens, maxlen = _pack_pwms(pwms, lens)
    K = len(lens)
    out = np.zeros(K, np.float32)
    _check(c._h, _lib.lib().cdlgb_pvalue_thresholds(c._h, ptr(arr, C.c_float), ptr(lens, C.c_int32), K,
                                                    maxlen, float(pval), ptr(out, C.c_float)))
    return out


def non_overlap_scan(c: CDL, positions, scores, lens, use_comp=None):
    """non_overlap_scan!'s selection (src/SEARCH/scan.jl:123-174; without use_comp,
    non_overlapping_scan_bg! :48-87) on the output of overlapping_scan: per sequence the
    highest-scoring motifs whose spans do not overlap are kept, the other entries are
    deleted (position 0).  Returns new (positions, scores, use_comp) arrays (N, K); the
    count re-evaluation that follows in the reference is count_matrices /
    posdicts2pfms on the kept positions."""
    pos = np.array(positions, np.int32, copy=True, order="C")
    sc = np.array(scores, np.float32, copy=True, order="C")
    uc = None if use_comp is None else np.array(use_comp, np.uint8, copy=True, order="C")
    lens = np.ascontiguousarray(lens, np.int32)
    K = len(lens)
    if pos.shape != (c.N, K) or sc.shape != (c.N, K):
        raise ValueError("positions / scores must be (N, K)")
    _check(c._h, _lib.lib().cdlgb_select_nonoverlapping(c._h, ptr(pos, C.c_int32), ptr(sc, C.c_float),
                                                        ptr(uc, C.c_uint8), ptr(lens, C.c_int32), K))
    return pos, sc, uc


def count_matrices(c: CDL, positions: np.ndarray, lens, use_comp=None):
    """Integer count matrices of the windows at ``positions`` (N, K) (1-based, 0 = none),
    reverse-complemented where use_comp != 0.  Returns (counts int32 (K, maxlen, 4) ==
    Julia (4, maxlen, K), nseq int32 (K,))."""
    pos = np.ascontiguousarray(positions, np.int32)
    lens = np.ascontiguousarray(lens, np.int32)
    K = len(lens)
    maxlen = int(lens.max())
    uc = None if use_comp is None else np.ascontiguousarray(use_comp, np.uint8)
    counts = np.zeros((K, maxlen, 4), np.int32)
    nseq = np.zeros(K, np.int32)
    _check(c._h, _lib.lib().cdlgb_count_pfms(c._h, ptr(pos, C.c_int32), ptr(uc, C.c_uint8),
                                             ptr(lens, C.c_int32), K, maxlen,
                                             ptr(counts, C.c_int32), ptr(nseq, C.c_int32)))
    return counts, nseq


def posdicts2pfms(c: CDL, positions: np.ndarray, lens, use_comp=None, pseudocounts_r=0.0295,
                  pseudo_count=5.0, smoothing=True, less_pseudocount=False) -> list:
    """posdicts2pfms (src/SEARCH/helpers.jl:59-96): count matrices on the GPU, the
    float32 normalisation on the host.  Returns a list of (4, w_k) float32 PFMs."""
    counts, nseq = count_matrices(c, positions, lens, use_comp)
    lens = np.ascontiguousarray(lens, np.int32)
    K, maxlen = len(lens), int(lens.max())
    out = np.zeros((K, maxlen, 4), np.float32)
    st = _lib.lib().cdlgb_counts_to_pfms(ptr(counts, C.c_int32), ptr(nseq, C.c_int32),
                                         ptr(lens, C.c_int32), K, maxlen, float(pseudocounts_r),
                                         float(pseudo_count), 1 if smoothing else 0,
                                         1 if less_pseudocount else 0, ptr(out, C.c_float))
    if st != 0:
        raise CDLGBError(st, "counts_to_pfms")
    return [out[k, : lens[k], :].T.copy() for k in range(K)]


_BG = (0.25, 0.25, 0.25, 0.25)


def extension(c: CDL, positions, lens, use_comp=None, bg=_BG, pseudocount=5.0,
              perc_no_less_than=0.95, ic_extension_thresh=0.075):
    """extension! (src/SEARCH/extend.jl:31-81 without use_comp, :122-173 with it) for
    every motif at once on the GPU.  positions (N, K) 1-based, 0 = none; use_comp (N, K)
    or None.  Returns (positions, lens, dec, inc): the new starts (0 for sequences
    dropped by the extension), the new lengths and the columns added on each side."""
    pos = np.array(positions, np.int32, copy=True, order="C")
    ln = np.array(lens, np.int32, copy=True)
    K = len(ln)
    if pos.shape != (c.N, K):
        raise ValueError("positions must be (N, K)")
    uc = None if use_comp is None else np.ascontiguousarray(use_comp, np.uint8)
    bgv = np.ascontiguousarray(bg, np.float32)
    dec = np.zeros(K, np.int32)
    inc = np.zeros(K, np.int32)
    _check(c._h, _lib.lib().cdlgb_extend_positions(
        c._h, ptr(pos, C.c_int32), ptr(uc, C.c_uint8), ptr(ln, C.c_int32), K, ptr(bgv, C.c_float),
        float(pseudocount), float(perc_no_less_than), float(ic_extension_thresh),
        ptr(dec, C.c_int32), ptr(inc, C.c_int32)))
    return pos, ln, dec, inc


def extend(c: CDL, positions, lens, filter_size: int, use_comp=None, bg=_BG, pseudocount=5.0,
           perc_no_less_than=0.95, ic_extension_thresh=0.075, pseudocounts_r=0.0295,
           smoothing=True, re_evaluate_pfm=True) -> dict:
    """extend! (src/SEARCH/extend.jl:175-211): extension of every motif, then the motifs
    with no positions left or a length <= filter_size + 2 are dropped, then (with
    re_evaluate_pfm, the reference's default) the PFMs are re-evaluated from the new
    positions by posdicts2pfms.  Returns {"positions" (N, K'), "lens", "use_comp",
    "pfms" (list or None), "keep" (bool (K,))}."""
    pos, ln, _, _ = extension(c, positions, lens, use_comp, bg, pseudocount, perc_no_less_than,
                              ic_extension_thresh)
    keep = (pos > 0).any(axis=0) & (ln > filter_size + 2)
    kept = np.flatnonzero(keep)
    pos = pos.take(kept, axis=1)          # (a C-order copy; faster than a boolean column index)
    ln = ln[keep]
    uc = None if use_comp is None else np.asarray(use_comp).take(kept, axis=1)
    pfms = None
    if re_evaluate_pfm:
        pfms = posdicts2pfms(c, pos, ln, uc, pseudocounts_r, pseudocount, smoothing) if len(ln) else []
    return {"positions": pos, "lens": ln, "use_comp": uc, "pfms": pfms, "keep": keep}


def trim_pfms(pfms, bg=_BG, mask_len=(8, 4, 2, 1), mask_thresh=(0.625, 0.525, 0.345, 0.2)):
    """trim_this_pfm_by_masking! (src/SEARCH/trim.jl:1-36) for a list of (4, w) PFMs,
    in the library's host code.  Returns (front, back) int32 arrays: the columns to
    trim at each end."""
    K = len(pfms)
    lens = np.array([np.asarray(p).shape[1] for p in pfms], np.int32)
    maxlen = max(1, int(lens.max()) if K else 1)
    arr = np.zeros((K, maxlen, 4), np.float32)
    for k, p in enumerate(pfms):
        arr[k, : lens[k], :] = np.asarray(p, np.float32).T
    bgv = np.ascontiguousarray(bg, np.float32)
    ml = np.ascontiguousarray(mask_len, np.int32)
    mt = np.ascontiguousarray(mask_thresh, np.float32)
    front = np.zeros(K, np.int32)
    back = np.zeros(K, np.int32)
    if K == 0:
        return front, back
    st = _lib.lib().cdlgb_trim_pfms(ptr(arr, C.c_float), ptr(lens, C.c_int32), K, maxlen,
                                    ptr(bgv, C.c_float), ptr(ml, C.c_int32), ptr(mt, C.c_float),
                                    len(ml), ptr(front, C.c_int32), ptr(back, C.c_int32))
    if st != 0:
        raise CDLGBError(st, "trim_pfms")
    return front, back


def masked_trim(pfms, filter_size: int, positions=None, use_comp=None, bg=_BG,
                mask_len=(8, 4, 2, 1), mask_thresh=(0.625, 0.525, 0.345, 0.2),
                after_merged=False, update_positions=True, c: CDL | None = None,
                pval_thresh=2.7e-4) -> dict:
    """masked_trim! (src/SEARCH/trim.jl:38-77): every PFM trimmed by masking, every
    position moved by the columns trimmed at the front (at the back for
    reverse-complemented entries when after_merged), then the motifs of length
    <= filter_size + 1 or without positions dropped.  With a context ``c`` the
    re-evaluation that follows in the reference (pwms = pfm2pwm, thresh = get_thresh at
    pval_thresh) is done too.  use_comp is returned unfiltered, as the reference leaves
    it (trim.jl:71-74).  Returns {"pfms", "lens", "positions", "keep", "front", "back",
    "pwms", "thresh"}."""
    front, back = trim_pfms(pfms, bg, mask_len, mask_thresh)
    new = [np.asarray(p, np.float32)[:, f: np.asarray(p).shape[1] - b]
           if f + b < np.asarray(p).shape[1] else np.zeros((4, 0), np.float32)
           for p, f, b in zip(pfms, front, back)]
    pos = None
    if positions is not None:
        # every entry (position > 0) moves by its motif's front trim, or by its back
        # trim when reverse-complemented after merging (trim.jl:47-59)
        pos = np.array(positions, np.int32, copy=True)
        if after_merged and use_comp is not None:
            shift = np.where(np.asarray(use_comp) != 0, back[None, :], front[None, :]).astype(np.int32)
        else:
            shift = front[None, :]
        pos += (pos > 0).astype(np.int32) * shift
    keep = np.array([p.shape[1] > filter_size + 1 for p in new], bool)
    if pos is not None:
        keep &= (pos > 0).any(axis=0)
    new = [p for p, kk in zip(new, keep) if kk]
    lens = np.array([p.shape[1] for p in new], np.int32)
    out = {"pfms": new, "lens": lens, "keep": keep, "front": front, "back": back,
           "positions": (pos.take(np.flatnonzero(keep), axis=1) if (pos is not None and update_positions)
                         else None),
           "use_comp": use_comp, "pwms": None, "thresh": None}
    if c is not None and len(new):
        pwms = [pfm2pwm(p, bg) for p in new]
        out["pwms"] = pwms
        out["thresh"] = get_thresh(c, pwms, pval_thresh)
    return out


def scores_reevaluation(c: CDL, pwms, positions, lens=None) -> np.ndarray:
    """scores_reevaluation (src/SEARCH/helpers.jl:151-172) on the GPU: the Float32 score
    of every entry's forward window.  pwms: list of (4, w); positions (N, K).
    Returns scores (N, K), 0 where there is no entry."""
    arr, ln, maxlen = _pack_pwms(pwms, lens)
    K = len(ln)
    pos = np.ascontiguousarray(positions, np.int32)
    if pos.shape != (c.N, K):
        raise ValueError("positions must be (N, K)")
    out = np.zeros((c.N, K), np.float32)
    _check(c._h, _lib.lib().cdlgb_rescore_positions(c._h, ptr(arr, C.c_float), ptr(pos, C.c_int32),
                                                    ptr(ln, C.c_int32), K, maxlen, ptr(out, C.c_float)))
    return out


def fisher_evalues(hits, hits_bg, N: int) -> np.ndarray:
    """filter_using_evalue!'s e-values (src/SEARCH/e_value_filter.jl:15-23):
    K * pvalue(FisherExactTest(a, N, b, N)) per motif, in the library's host code."""
    a = np.ascontiguousarray(hits, np.int32)
    b = np.ascontiguousarray(hits_bg, np.int32)
    out = np.zeros(len(a), np.float64)
    if len(a) == 0:
        return out
    st = _lib.lib().cdlgb_fisher_evalues(ptr(a, C.c_int32), ptr(b, C.c_int32), len(a), int(N),
                                         ptr(out, C.c_double))
    if st != 0:
        raise CDLGBError(st, "fisher_evalues")
    return out


def filter_using_evalue(c: CDL, pwms, thresh, positions, lens=None, cpu=False, non_overlap=False,
                        e_value_thresh_1=0.5, e_value_thresh_2=1e-3,
                        get_evalues_only=False):
    """filter_using_evalue! (src/SEARCH/e_value_filter.jl:1-44) on c's background
    (make it first with c.make_background()): the motifs are scanned on the background
    (cpu=False: the forward GPU scan of scan_w_gpu!; cpu=True: the two-strand scan of
    overlapping_scan_bg!, then with non_overlap the selection of
    non_overlapping_scan_bg!), the sequences hit in the data (positions (N, K), 0 = none)
    and in the background are compared by Fisher's exact test, and a motif passes when
    its e-value is below the threshold (Float32 e_value_thresh_2 with cpu, else
    e_value_thresh_1) and its length is above 5.  Returns the e-values when
    get_evalues_only, else {"evalues", "keep", "hits", "hits_bg"}."""
    _, ln, _ = _pack_pwms(pwms, lens)
    with c.on_background():
        if not cpu:
            bg_pos = scan_w_gpu(c, pwms, thresh, ln)
        else:
            bg_pos, bg_sc, _ = overlapping_scan(c, pwms, thresh, ln)
            if non_overlap:
                bg_pos, _, _ = non_overlap_scan(c, bg_pos, bg_sc, ln, None)
    hits = (np.asarray(positions) > 0).sum(axis=0).astype(np.int32)
    hits_bg = (bg_pos > 0).sum(axis=0).astype(np.int32)
    ev = fisher_evalues(hits, hits_bg, c.N)
    if get_evalues_only:
        return ev
    thr = float(np.float32(e_value_thresh_2 if cpu else e_value_thresh_1))
    keep = (ev < thr) & (ln > 5)
    return {"evalues": ev, "keep": keep, "hits": hits, "hits_bg": hits_bg}


# ---------------------------------------------------------------------------- code -> counts
class ActivationRecord:
    """activation_record (src/SETUP/SEARCH_setup.jl:6-57), device resident: the codes of
    `T` trainings over N sequences of L bases with M filters each."""

    def __init__(self, N: int, L: int, M: int, T: int = 2, device: int = 0):
        h = C.c_void_p()
        st = _lib.lib().cdlgb_ar_create(int(N), int(L), int(M), int(T), int(device), C.byref(h))
        if st != 0:
            raise CDLGBError(st, _lib.lib().cdlgb_ar_last_error(None).decode())
        self._h = h
        self.N, self.L, self.M, self.T = N, L, M, T

    def _check(self, st):
        if st != 0:
            msg = _lib.lib().cdlgb_ar_last_error(self._h)
            raise CDLGBError(st, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().cdlgb_ar_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        """(uinds, training_num, filter_lengths) of the recorded filters, 1-based."""
        K = C.c_int32()
        self._check(_lib.lib().cdlgb_ar_info(self._h, C.byref(K), None, None, None, 0))
        k = K.value
        u, t, f = (np.zeros(max(k, 1), np.int32) for _ in range(3))
        self._check(_lib.lib().cdlgb_ar_info(self._h, C.byref(K), ptr(u, C.c_int32), ptr(t, C.c_int32),
                                             ptr(f, C.c_int32), max(k, 1)))
        return u[:k], t[:k], f[:k]


def record_training_result(c: CDL, thresh: float, ar: ActivationRecord, train_num: int,
                           filter_size: int) -> int:
    """record_training_result! (src/SEARCH/store.jl:1-40): returns the number of
    filters added."""
    added = C.c_int32()
    ar._check(_lib.lib().cdlgb_ar_record(ar._h, c._h, float(thresh), int(train_num),
                                         int(filter_size), C.byref(added)))
    return added.value


def get_spatial_info(ar: ActivationRecord):
    """get_spatial_info! (src/SEARCH/store.jl:121-144).  Returns numpy int32 arrays
    over (maxlen, K, K), non_over (L - minlen - 1, K, K), next_to (K, K), indexed
    [distance, fc, fr] (Julia [fr, fc, distance])."""
    u, t, f = ar.info()
    K = len(u)
    maxlen, minlen = int(f.max()), int(f.min())
    over = np.zeros((maxlen, K, K), np.int32)
    non_over = np.zeros((max(ar.L - minlen - 1, 0), K, K), np.int32)
    next_to = np.zeros((K, K), np.int32)
    ar._check(_lib.lib().cdlgb_ar_topology(ar._h, ptr(over, C.c_int32), ptr(non_over, C.c_int32),
                                           ptr(next_to, C.c_int32)))
    return over, non_over, next_to


def select_pairs(over: np.ndarray, count_threshold: int) -> np.ndarray:
    """findall(over .> count_threshold) in Julia order (extractions.jl:24-26): rows of
    1-based (fr, fc, overlap)."""
    o, fc, fr = np.nonzero(np.asarray(over) > count_threshold)
    order = np.lexsort((fr, fc, o))
    return np.stack([fr[order] + 1, fc[order] + 1, o[order] + 1], axis=1).astype(np.int32)


def get_pair_pfms(ar: ActivationRecord, c: CDL, over: np.ndarray, count_threshold: int,
                  filter_size: int):
    """get_pair_pfms! (src/SEARCH/extractions.jl:18-114) without the p-value thresholds:
    returns (pairs (P, 3), span_lens (P,), pfms list of (4, span) float32)."""
    pairs = np.ascontiguousarray(select_pairs(over, count_threshold))
    P = len(pairs)
    if P == 0:
        return pairs, np.zeros(0, np.int32), []
    max_span = 2 * filter_size - 1
    out = np.zeros((max_span, 4, P), np.float32)
    spans = np.zeros(P, np.int32)
    ar._check(_lib.lib().cdlgb_ar_pair_pfms(ar._h, c._h, ptr(pairs, C.c_int32), P, int(filter_size),
                                            ptr(out, C.c_float), ptr(spans, C.c_int32)))
    return pairs, spans, [out[: spans[p], :, p].T.copy() for p in range(P)]


def pfm2pwm(pfm, bg=(0.25, 0.25, 0.25, 0.25)):
    """pfm2pwm (src/SEARCH/helpers.jl:12-13): log2(pfm ./ bg) in the pfm's precision."""
    pfm = np.asarray(pfm)
    return np.log2(pfm / np.asarray(bg, pfm.dtype).reshape(4, 1))


def pwm_complement(pwm):
    """pwm_complement = reverse (src/SEARCH/helpers.jl:16)."""
    return np.asarray(pwm)[::-1, ::-1].copy()


def transfac_text(pfm, reverse_complement: bool = False) -> str:
    """One transfac file body as save_pfms_as_transfac writes it."""
    p = np.ascontiguousarray(np.asarray(pfm, np.float32).T)   # (w, 4) == Julia (4, w)
    w = p.shape[0]
    L = _lib.lib()
    n = L.cdlgb_transfac_format(ptr(p, C.c_float), w, 1 if reverse_complement else 0, None, 0)
    if n < 0:
        raise CDLGBError(int(n), "transfac_format")
    buf = C.create_string_buffer(int(n) + 1)
    L.cdlgb_transfac_format(ptr(p, C.c_float), w, 1 if reverse_complement else 0, buf, n + 1)
    return buf.value.decode()


def save_pfms_as_transfac(logo_folder: str, pfms: list, sort_perm=None):
    """save_pfms_as_transfac (src/SAVE/save_learned_results.jl:184-217) without the
    weblogo calls (an external tool): writes d{i}.transfac and d{i}_c.transfac."""
    os.makedirs(logo_folder, exist_ok=True)
    sort_perm = list(range(1, len(pfms) + 1)) if sort_perm is None else list(sort_perm)
    for i, ind in enumerate(sort_perm, start=1):
        with open(os.path.join(logo_folder, f"d{i}.transfac"), "w") as f:
            f.write(transfac_text(pfms[ind - 1], False))
        with open(os.path.join(logo_folder, f"d{i}_c.transfac"), "w") as f:
            f.write(transfac_text(pfms[ind - 1], True))
