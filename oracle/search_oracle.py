"""CPU oracle for CDLmotif's code -> counts -> PWM-scan stage.

TEST INFRASTRUCTURE ONLY (see cdl_oracle.py for the rules): the checker for the
CUDA scan/count kernels, never the product path.

Parity status: **parity unpinned** against reference-produced vectors (the
reference's test suite is empty); the FP32 operation order of each scan path is
restated exactly so that scan scores, positions and integer counts are compared
bit for bit.

Layouts (C-order numpy == Julia column-major bytes):
  one-hot data   Julia (4L, N)            -> numpy (N, 4L)
  pwms           Julia (K, 4, maxlen)     -> numpy (maxlen, 4, K)
  positions      Julia Dict per motif     -> numpy int32 (N, K) Julia (K, N), 0 = none
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


# ----------------------------------------------------------------------------------
# a20: scan_w_gpu! / greedy_search!  (src/SEARCH/scan.jl:176-239)
# ----------------------------------------------------------------------------------
def greedy_search(pwms_k4w: np.ndarray, data: np.ndarray, lens: np.ndarray,
                  thresh: np.ndarray) -> np.ndarray:
    """src/SEARCH/scan.jl:223-239.  Returns pos_scores as numpy (K, N, L) float32
    (index [k, n, l]).  Each score is accumulated in FP32 starting from the zeroed
    buffer, position-major (ind outer, nucleotide a inner), one rounded multiply and
    one rounded add per term (no FMA), then replaced by 0 unless > thresh[k]."""
    K = pwms_k4w.shape[0]
    N, L4 = data.shape
    L = L4 // 4
    onehot = data.reshape(N, L, 4).astype(f32)
    out = np.zeros((K, N, L), dtype=f32)
    for k in range(K):
        w = int(lens[k])
        nl = L - w + 1
        if nl <= 0:
            continue
        s = np.zeros((N, nl), dtype=f32)
        for ind in range(w):
            for a in range(4):
                p = f32(pwms_k4w[k, a, ind])
                s = (s + (p * onehot[:, ind:ind + nl, a]).astype(f32)).astype(f32)
        s = np.where(s > f32(thresh[k]), s, f32(0.0)).astype(f32)
        out[k, :, :nl] = s
    return out


def scan_w_gpu_positions(pwms_k4w, data, lens, thresh) -> np.ndarray:
    """src/SEARCH/scan.jl:189-205: argmax over positions (first maximum, Julia
    ``argmax(dims=3)``), then a 1-based argmax of 1 becomes 0 = "not found"
    (the reference drops a true best hit at position 1 as well).  Returns int32 (K, N)
    1-based positions, 0 = none."""
    ps = greedy_search(pwms_k4w, data, lens, thresh)
    am = np.argmax(ps, axis=2) + 1          # numpy argmax also returns the first maximum
    am[am == 1] = 0
    return am.astype(np.int32)


# ----------------------------------------------------------------------------------
# a21: scan_n / overlapping_scan!  (src/SEARCH/scan.jl:10-21, 89-121)
# ----------------------------------------------------------------------------------
def pwm_complement(pwm_4w: np.ndarray) -> np.ndarray:
    """src/SEARCH/helpers.jl:16 -- ``reverse`` of a matrix reverses both dims."""
    return pwm_4w[::-1, ::-1].copy()


def scan_n_all(onehot_nl4: np.ndarray, pwm_4w: np.ndarray):
    """Vectorised src/SEARCH/scan.jl:10-21 over all sequences: FP32 scores summed
    nucleotide-major (``for j=1:4, k=1:len``), strict ``>`` so the first maximum wins,
    starting from (-1, -Inf).  Returns (idx int32 (N,), score float32 (N,))."""
    N, L, _ = onehot_nl4.shape
    w = pwm_4w.shape[1]
    nl = L - w + 1
    if nl <= 0:
        return np.full(N, -1, np.int32), np.full(N, -np.inf, f32)
    s = np.zeros((N, nl), dtype=f32)
    for j in range(4):
        for k in range(w):
            p = f32(pwm_4w[j, k])
            s = (s + (p * onehot_nl4[:, k:k + nl, j]).astype(f32)).astype(f32)
    # sequential strict '>' from -Inf == first index of the maximum, NaN never wins
    best = np.full(N, -np.inf, f32)
    idx = np.full(N, -1, np.int32)
    for i in range(nl):
        gt = s[:, i] > best
        best = np.where(gt, s[:, i], best)
        idx = np.where(gt, i + 1, idx)
    return idx.astype(np.int32), best.astype(f32)


def overlapping_scan(data: np.ndarray, pwms: list, lens, thresh):
    """src/SEARCH/scan.jl:89-121: both strands, forward kept on ties (score >= score_c),
    a hit recorded only if its score > thresh[k].  Returns (pos int32 (K,N) 0=none,
    score float32 (K,N), use_comp uint8 (K,N))."""
    N, L4 = data.shape
    L = L4 // 4
    onehot = data.reshape(N, L, 4).astype(f32)
    K = len(pwms)
    pos = np.zeros((K, N), np.int32)
    score = np.zeros((K, N), f32)
    comp = np.zeros((K, N), np.uint8)
    for k in range(K):
        pwm = np.asarray(pwms[k], dtype=f32)[:, : int(lens[k])]
        i_f, s_f = scan_n_all(onehot, pwm)
        i_c, s_c = scan_n_all(onehot, pwm_complement(pwm))
        fwd = s_f >= s_c
        s = np.where(fwd, s_f, s_c)
        i = np.where(fwd, i_f, i_c)
        keep = s > f32(thresh[k])
        pos[k] = np.where(keep, i, 0)
        score[k] = np.where(keep, s, f32(0))
        comp[k] = np.where(keep & ~fwd, 1, 0)
    return pos, score, comp


# ----------------------------------------------------------------------------------
# a22: posdicts2pfms (src/SEARCH/helpers.jl:59-96)
# ----------------------------------------------------------------------------------
def read_fasta_onehot(text: bytes, max_entries: int = 10000):
    """reading + read_fasta (src/LOAD/read.jl:2-28) and data_2_dummy
    (src/LOAD/to_dummy.jl:27-38): records are the '>'-separated chunks, the header line
    of each dropped and the remaining lines joined (only '\n' removed); records with
    'N'/'n' are dropped, the first max_entries kept and upper-cased; the one-hot matrix
    (N, 4L) float32 has a zero row for records whose length differs from the first one's
    (uninitialised in the reference).  Returns (onehot, reads)."""
    s = text.decode("latin-1") if isinstance(text, (bytes, bytearray)) else text
    reads = []
    for chunk in s.split(">"):
        if chunk:
            r = "".join(chunk.split("\n")[1:])
            if "N" not in r and "n" not in r:
                reads.append(r)
    reads = [r.upper() for r in reads[:max_entries]]
    L = len(reads[0])
    out = np.zeros((len(reads), 4 * L), np.float32)
    code = {"A": 0, "C": 1, "G": 2, "T": 3}
    for n, r in enumerate(reads):
        if len(r) != L:
            continue
        for i, ch in enumerate(r):
            out[n, 4 * i + code[ch]] = 1.0
    return out, reads


def pvalue2score(pwm_4m, pval: float, eps: float = 1e-1, bg=(0.25, 0.25, 0.25, 0.25)):
    """pvalue2score (src/SEARCH/PWM_Touzet.jl:199-217) in exact rational arithmetic
    (the reference's Double64 is exact here: every rounded entry is an integer multiple
    of the Float64 eps, every probability a power of two), then get_thresh's Float32
    (helpers.jl:99).  Literal restatement: min_score_range column order, round_pwm,
    score_distribution(pwm_eps, worst_score(pwm_eps), Inf, bg) and find_largest_alpha."""
    import math
    from fractions import Fraction as Fr
    P = [[Fr(float(x)) for x in row] for row in np.asarray(pwm_4m, np.float32)]
    m = len(P[0])
    e = Fr(eps)
    rng = [max(P[j][i] for j in range(4)) - min(P[j][i] for j in range(4)) for i in range(m)]
    order = sorted(range(m), key=lambda i: -rng[i])          # stable, as sortperm(rev=true)
    R = [[math.floor(P[j][i] / e) * e for i in order] for j in range(4)]
    alpha = sum(min(R[j][i] for j in range(4)) for i in range(m))
    bgf = [Fr(b) for b in bg]
    Q = {Fr(0): Fr(1)}
    for i in range(m):
        bs = sum(max(R[j][ii] for j in range(4)) for ii in range(i + 1, m))
        Qn = {}
        for score in sorted(Q):
            for j in range(4):
                t = score + R[j][i]
                if alpha - bs <= t:                              # t <= beta - ws with beta = Inf
                    Qn[t] = Qn.get(t, Fr(0)) + Q[score] * bgf[j]
        Q = Qn
    q_sum = sum(Q.values())
    largest = None
    for k in sorted(Q):
        if q_sum >= Fr(pval):
            largest = k
        else:
            return np.float32(float(k))
        q_sum -= Q[k]
    return np.float32(float(largest))


def non_overlap_select(pos: np.ndarray, score: np.ndarray, use_comp, lens):
    """non_overlap_scan! (src/SEARCH/scan.jl:123-174; non_overlapping_scan_bg! :48-87 is
    the same loop without use_comp).  pos, score, use_comp are (N, K) == Julia (K, N)
    with pos 0 = no entry for (k, n).  Per sequence: repeatedly take the motif of largest
    score (Julia argmax: the first maximum; scores of motifs without an entry, and of
    motifs already taken, count as 0) until that largest score is 0; keep it when its
    span [p, p + len - 1] meets no kept span.  Entries not kept are deleted (pos, score,
    use_comp set to 0).  Returns new (pos, score, use_comp) arrays."""
    pos = np.array(pos, np.int32, copy=True)
    score = np.array(score, np.float32, copy=True)
    uc = None if use_comp is None else np.array(use_comp, np.uint8, copy=True)
    N, K = pos.shape
    lens = [int(x) for x in lens]
    for n in range(N):
        spans = []
        keep = [False] * K
        sc = [float(score[n, k]) if pos[n, k] != 0 else 0.0 for k in range(K)]
        ps = [int(pos[n, k]) for k in range(K)]
        best = int(np.argmax(np.array(sc, np.float32)))
        while sc[best] != 0:
            pm, pme = ps[best], ps[best] + lens[best] - 1
            hit = False
            for (p, l) in spans:
                pe = p + l - 1
                if p <= pm <= pe or p <= pme <= pe or pm <= p <= pme or pm <= pe <= pme:
                    hit = True
            if not hit:
                keep[best] = True
                spans.append((ps[best], lens[best]))
            sc[best] = 0.0
            best = int(np.argmax(np.array(sc, np.float32)))
        for k in range(K):
            if not keep[k] and pos[n, k] != 0:
                pos[n, k] = 0
                score[n, k] = 0
                if uc is not None:
                    uc[n, k] = 0
    return pos, score, uc


def count_matrices(data: np.ndarray, pos: np.ndarray, use_comp, lens) -> tuple:
    """The MSA column sums of posdicts2pfms (helpers.jl:73-89) as integers: for every
    motif k and sequence n with pos[k,n] > 0, add the one-hot window starting at base
    pos[k,n] (reverse-complemented, ``submat_comlement``, when use_comp[k,n]).
    Returns (counts int32 (K, maxlen, 4) == Julia (4, maxlen, K), nseq int32 (K,))."""
    N, L4 = data.shape
    L = L4 // 4
    onehot = data.reshape(N, L, 4)
    K = pos.shape[0]
    maxlen = int(max(lens))
    counts = np.zeros((K, maxlen, 4), np.int64)
    nseq = np.zeros(K, np.int32)
    for k in range(K):
        w = int(lens[k])
        for n in range(N):
            p = int(pos[k, n])
            if p <= 0:
                continue
            win = onehot[n, p - 1:p - 1 + w, :]
            if use_comp is not None and use_comp[k, n]:
                win = win[::-1, ::-1]
            counts[k, :w, :] += win.astype(np.int64)
            nseq[k] += 1
    return counts.astype(np.int32), nseq


def counts_to_pfms(counts, nseq, lens, pseudocounts_r=0.0295, pseudo_count=5.0,
                   smoothing=True, less_pseudocount=False) -> list:
    """helpers.jl:66,87-88 in FP32: ps = r*n (smoothing) or a fixed 5 / 0.1;
    pfm = (count + ps) / (n + 4*ps)."""
    pfms = []
    for k in range(len(lens)):
        n = int(nseq[k])
        if smoothing:
            ps = f32(f32(pseudocounts_r) * f32(n))
        else:
            ps = f32(0.1) if less_pseudocount else f32(pseudo_count)
        den = f32(f32(n) + f32(f32(4) * ps))
        c = counts[k, : int(lens[k]), :].T.astype(f32)       # (4, w)
        pfms.append(((c + ps).astype(f32) / den).astype(f32))
    return pfms


# ----------------------------------------------------------------------------------
# (f) motif refinement: extend! / masked_trim! / scores_reevaluation
# ----------------------------------------------------------------------------------
def _log2_f32(q) -> np.float32:
    """Float32 log2 correctly rounded: evaluated in float64 and rounded (the reference's
    Float32 log2 evaluates in Float64 and rounds too)."""
    return f32(np.log2(np.float64(q)))


def ic_col_single(col, bg) -> np.float32:
    """get_ic_col_single (src/SEARCH/helpers.jl:127-133): s += p[i] * log2(p[i] / bg[i])
    in Float32, i = 1..4 in order."""
    s = f32(0)
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(4):
            p = f32(col[i])
            s = f32(s + f32(p * _log2_f32(f32(p / f32(bg[i])))))
    return s


_DUMMY_COMP = {(1, 0, 0, 0): (0, 0, 0, 1), (0, 1, 0, 0): (0, 0, 1, 0),
               (0, 0, 1, 0): (0, 1, 0, 0), (0, 0, 0, 1): (1, 0, 0, 0)}


def _dummy_comp(v):
    """dummy_comp (src/SEARCH/helpers.jl:18-41): a Dict lookup, so anything but one of
    the four one-hot vectors raises KeyError."""
    return np.array(_DUMMY_COMP[tuple(int(x) if float(x) in (0.0, 1.0) else x for x in v)], f32)


def extension(data: np.ndarray, pos_col, mlen: int, comp_col, bg=(0.25,) * 4, pseudocount=5.0,
              perc_no_less_than=0.95, ic_extension_thresh=0.075):
    """extension! for one motif (src/SEARCH/extend.jl:31-81 when comp_col is None,
    :122-173 otherwise), restated statement by statement with its per-sequence
    `included` flags.  data (N, 4L) one-hot; pos_col (N,) 1-based positions, 0 = not a
    key; comp_col (N,) use_comp flags or None.  Returns (new pos_col, new length,
    dec, inc).  The reference's num_included is decremented only inside
    explore_sides! (a local copy), so the usage bound of :74 / :165 compares the
    unchanged entry count.  Raises RuntimeError after 2L + 4 passes (the reference
    does not return then) and KeyError where dummy_comp does."""
    N, L4 = data.shape
    L = L4 // 4
    keys = [n for n in range(N) if pos_col[n] != 0]
    P = {n: int(pos_col[n]) for n in keys}
    C = None if comp_col is None else {n: bool(comp_col[n]) for n in keys}
    ps = f32(pseudocount)
    thr = f32(ic_extension_thresh)
    len_pos = len(keys)
    dec = inc = 0
    included = [True] * len_pos
    num_included = len_pos
    usage_lowerbdd = int(np.floor(f32(f32(perc_no_less_than) * f32(len_pos))))
    explore_left = explore_right = True
    len_inc = 0

    def explore_sides(offset, right):
        this_col = np.zeros(4, f32)
        inc_right = mlen - 1 + offset
        to_exclude = []
        for ind, k in enumerate(keys):
            if not included[ind]:
                continue
            if C is None:
                pos = P[k] + inc_right if right else P[k] - offset
            else:
                pos = P[k] + inc_right if ((right and not C[k]) or (not right and C[k])) else P[k] - offset
            if pos < 1 or pos > L:
                to_exclude.append(ind)
                continue
            dat = data[k, 4 * (pos - 1):4 * pos].astype(f32)
            if C is not None and C[k]:
                dat = _dummy_comp(dat)
            this_col = (this_col + dat).astype(f32)
        tot = f32(f32(f32(this_col[0] + this_col[1]) + this_col[2]) + this_col[3])
        col = ((this_col + ps).astype(f32) / f32(tot + f32(f32(4) * ps))).astype(f32)
        return ic_col_single(col, bg), to_exclude

    passes = 0
    while True:
        passes += 1
        if passes > 2 * L + 4:
            raise RuntimeError("extension does not terminate")
        if explore_left:
            ic, ex = explore_sides(dec + 1, False)
            if ic <= thr:
                explore_left = False
            else:
                for i in ex:
                    included[i] = False
                len_inc += 1
                dec += 1
        if explore_right:
            ic, ex = explore_sides(inc + 1, True)
            if ic <= thr:
                explore_right = False
            else:
                for i in ex:
                    included[i] = False
                len_inc += 1
                inc += 1
        if not explore_left and not explore_right:
            break
        if num_included <= usage_lowerbdd:
            break
    out = np.array(pos_col, np.int32, copy=True)
    if dec > 0 or inc > 0:
        out[:] = 0
        for ind, k in enumerate(keys):
            if included[ind]:
                out[k] = P[k] - inc if (C is not None and C[k]) else P[k] - dec
    return out, mlen + len_inc, dec, inc


def extend_positions(data, pos, use_comp, lens, bg=(0.25,) * 4, pseudocount=5.0,
                     perc_no_less_than=0.95, ic_extension_thresh=0.075):
    """extension! for every motif (the loop of extend!, src/SEARCH/extend.jl:180-196).
    pos, use_comp (N, K) == Julia (K, N).  Returns (pos, lens, dec, inc)."""
    pos = np.array(pos, np.int32, copy=True)
    K = pos.shape[1]
    lens_out = np.array(lens, np.int32, copy=True)
    dec = np.zeros(K, np.int32)
    inc = np.zeros(K, np.int32)
    for k in range(K):
        cc = None if use_comp is None else use_comp[:, k]
        pos[:, k], lens_out[k], dec[k], inc[k] = extension(
            data, pos[:, k], int(lens[k]), cc, bg, pseudocount, perc_no_less_than,
            ic_extension_thresh)
    return pos, lens_out, dec, inc


def _median_f32(v):
    """median of a Float32 vector: NaN if any, else the middle value, or
    middle(a, b) = a/2 + b/2 of the two middle values."""
    v = np.asarray(v, f32)
    if np.any(np.isnan(v)):
        return f32(np.nan)
    v = np.sort(v)
    n = len(v)
    if n % 2:
        return v[n // 2]
    return f32(f32(v[n // 2 - 1] / f32(2)) + f32(v[n // 2] / f32(2)))


def ic_cols(pfm, bg=(0.25,) * 4) -> np.ndarray:
    """get_ic_col_multiple (src/SEARCH/helpers.jl:135-138): per column
    ((s1 + s2) + s3) + s4, s_a = p * log2(p / bg[a]) in Float32."""
    pfm = np.asarray(pfm, f32)
    return np.array([ic_col_single(pfm[:, j], bg) for j in range(pfm.shape[1])], f32)


def trim_pfm_by_masking(pfm, bg=(0.25,) * 4, mask_len=(8, 4, 2, 1),
                        mask_thresh=(0.625, 0.525, 0.345, 0.2)):
    """trim_this_pfm_by_masking! (src/SEARCH/trim.jl:1-36).  Returns (front, back)."""
    ic = ic_cols(pfm, bg)
    n = len(ic)
    trim = [False] * n
    for ml, mt in zip(mask_len, mask_thresh):
        mt = f32(mt)
        for i in range(0, n - ml + 1):
            if trim[i]:
                continue
            if _median_f32(ic[i:i + ml]) < mt:
                trim[i] = True
            else:
                break
        for j in range(n - 1, ml - 2, -1):
            if trim[j]:
                continue
            if _median_f32(ic[j - ml + 1:j + 1]) < mt:
                trim[j] = True
            else:
                break
    front = 0
    for t in trim:
        if not t:
            break
        front += 1
    back = 0
    for t in reversed(trim):
        if not t:
            break
        back += 1
    return front, back


def scores_reevaluation(data, pwms, pos, lens) -> np.ndarray:
    """scores_reevaluation (src/SEARCH/helpers.jl:151-172): per entry the sum of
    pwm .* the forward window (use_comp is not consulted), restated in memory order
    (base-major, nucleotide inner) with a rounded product and a rounded sum per term.
    pwms: list of (4, w); pos (N, K).  Returns scores (N, K), 0 where pos is 0."""
    N, L4 = data.shape
    K = pos.shape[1]
    out = np.zeros((N, K), f32)
    for k in range(K):
        w = int(lens[k])
        pw = np.asarray(pwms[k], f32)[:, :w]
        for n in range(N):
            p = int(pos[n, k])
            if p <= 0:
                continue
            win = data[n, 4 * (p - 1):4 * (p - 1 + w)].astype(f32)
            s = f32(0)
            for i in range(w):
                for a in range(4):
                    s = f32(s + f32(pw[a, i] * win[4 * i + a]))
            out[n, k] = s
    return out


# ----------------------------------------------------------------------------------
# (f) background + e-value filter (src/SETUP/LOAD_setup.jl:5-14,
#     src/SEARCH/e_value_filter.jl:1-65)
# ----------------------------------------------------------------------------------
_M64 = (1 << 64) - 1
_GOLDEN = 0x9E3779B97F4A7C15


def _mix64(z: int) -> int:
    """splitmix64's output function (Steele, Lea & Flood 2014)."""
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


class SplitMix:
    """Per-sequence splitmix64 stream: state = mix(seed ^ golden * (n + 1)); each draw
    adds the golden gamma and mixes; below(m) = ((z >> 32) * m) >> 32."""

    def __init__(self, seed: int, n: int):
        self.s = _mix64((seed ^ ((_GOLDEN * (n + 1)) & _M64)) & _M64)

    def below(self, m: int) -> int:
        self.s = (self.s + _GOLDEN) & _M64
        return ((_mix64(self.s) >> 32) * m) >> 32


def _fisher_yates(a: list, m: int, rng: SplitMix):
    for i in range(m - 1, 0, -1):
        j = rng.below(i + 1)
        a[i], a[j] = a[j], a[i]


def onehot_symbols(data: np.ndarray) -> np.ndarray:
    """(N, 4L) one-hot -> (N, L) symbols 0..3 (A C G T), 4 where the column is not a
    one-hot vector."""
    N, L4 = data.shape
    oh = data.reshape(N, L4 // 4, 4)
    ones = (oh == 1).sum(axis=2)
    zeros = (oh == 0).sum(axis=2)
    sym = np.argmax(oh == 1, axis=2).astype(np.int64)
    sym[~((ones == 1) & (zeros == 3))] = 4
    return sym


def klet_shuffle_seq(sym, k: int, rng: SplitMix) -> list:
    """k-let preserving shuffle of one symbol sequence (alphabet of 5): the Euler-path
    method of Altschul & Erickson with Wilson's random arborescence towards the last
    (k-1)-mer, in the draw order of the device kernel: the last exits of the vertices in
    increasing vertex order (loop-erased walks), then for each vertex in increasing
    order a Fisher-Yates shuffle of its other exits (all exits for the last vertex),
    then the walk from the first (k-1)-mer."""
    sym = [int(x) for x in sym]
    L = len(sym)
    if k == 1:
        a = list(sym)
        _fisher_yates(a, L, rng)
        return a
    E = L - k + 1
    if E <= 0:
        return list(sym)
    V = 5 ** (k - 1)
    v0 = 0
    for j in range(k - 1):
        v0 = v0 * 5 + sym[j]
    exits = [[] for _ in range(V)]
    u = v0
    for i in range(E):
        w = sym[i + k - 1]
        exits[u].append(w)
        u = (u * 5 + w) % V
    vend = u
    intree = [False] * V
    intree[vend] = True
    nxt = [0] * V
    for v in range(V):
        if not exits[v] or intree[v]:
            continue
        u = v
        while not intree[u]:
            nxt[u] = rng.below(len(exits[u]))
            u = (u * 5 + exits[u][nxt[u]]) % V
        u = v
        while not intree[u]:
            intree[u] = True
            u = (u * 5 + exits[u][nxt[u]]) % V
    for v in range(V):
        e = exits[v]
        m = len(e)
        if m == 0:
            continue
        if v != vend:
            e[nxt[v]], e[m - 1] = e[m - 1], e[nxt[v]]
            _fisher_yates(e, m - 1, rng)
        else:
            _fisher_yates(e, m, rng)
    out = sym[: k - 1]
    cur = [0] * V
    u = v0
    for _ in range(E):
        w = exits[u][cur[u]]
        cur[u] += 1
        out.append(w)
        u = (u * 5 + w) % V
    return out


def make_background(data: np.ndarray, k: int = 3, seed: int = 0) -> np.ndarray:
    """Every sequence of the (N, 4L) one-hot data k-let shuffled (sequence n with the
    stream SplitMix(seed, n)); symbol 4 becomes a zero column.  Returns (N, 4L)."""
    sym = onehot_symbols(data)
    N, L = sym.shape
    out = np.zeros((N, L, 4), np.float32)
    for n in range(N):
        s = klet_shuffle_seq(sym[n], k, SplitMix(seed, n))
        for i, x in enumerate(s):
            if x < 4:
                out[n, i, x] = 1.0
    return out.reshape(N, 4 * L)


def kmer_counts(sym_row, k: int) -> dict:
    out = {}
    for i in range(len(sym_row) - k + 1):
        key = tuple(int(x) for x in sym_row[i:i + k])
        out[key] = out.get(key, 0) + 1
    return out


def fisher_evalue_exact(a: int, b: int, N: int, K: int) -> float:
    """K * pvalue(FisherExactTest(a, N, b, N)) (src/SEARCH/e_value_filter.jl:19-23) from
    exact rationals: X ~ Hypergeometric(a + N, b + N, a + b), central two-sided
    p = min(1, 2 min(P(X <= a), P(X >= a)))."""
    from fractions import Fraction
    from math import comb
    r1, r2, c1 = a + N, b + N, a + b
    lo, hi = max(0, c1 - r2), min(c1, r1)
    den = comb(r1 + r2, c1)
    left = sum(comb(r1, j) * comb(r2, c1 - j) for j in range(lo, a + 1))
    right = sum(comb(r1, j) * comb(r2, c1 - j) for j in range(a, hi + 1))
    p = min(Fraction(1), 2 * min(Fraction(left, den), Fraction(right, den)))
    return float(p * K)


def pfm2pwm(pfm, bg=(0.25, 0.25, 0.25, 0.25)):
    """src/SEARCH/helpers.jl:12-13."""
    bgv = np.asarray(bg, dtype=np.asarray(pfm).dtype).reshape(4, 1)
    return np.log2(np.asarray(pfm) / bgv)


# ----------------------------------------------------------------------------------
# a17-a19: record_training_result!, topology_at_nth_pt!, get_pair_pfms!
# ----------------------------------------------------------------------------------
def record_codes(X_best: np.ndarray, gamma: int, L4: int) -> np.ndarray:
    """src/SEARCH/store.jl:15 -- X_best[gamma+1:4:gamma+L, :, :] -> codes (N, M, C)."""
    return X_best[:, :, gamma:gamma + L4:4].copy()


def activation_topology(start_pos: np.ndarray, train_num, fil_lens, C: int):
    """src/SEARCH/store.jl:64-107 and :121-144 with cover_starts == 1.
    start_pos: bool (N, K, C) (== Julia (C, K, N)).  Returns int32 arrays
    over (max_len, K, K), non_over (C-minlen-1, K, K), next_to (K, K) -- numpy index
    [.., fc, fr] matches Julia [fr, fc, ..]."""
    N, K, _ = start_pos.shape
    fil_lens = np.asarray(fil_lens)
    train_num = np.asarray(train_num)
    maxlen = int(fil_lens.max())
    CmFm1 = C - int(fil_lens.min()) - 1
    over = np.zeros((maxlen, K, K), np.int64)
    non_over = np.zeros((max(CmFm1, 0), K, K), np.int64)
    next_to = np.zeros((K, K), np.int64)
    for n in range(N):
        act = [(f, p + 1) for f in range(K) for p in np.nonzero(start_pos[n, f])[0]]
        for fr, pr_s in act:
            pr_e = pr_s + fil_lens[fr] - 1
            for fc, pc_s in act:
                if fr == fc or pr_s > pc_s or train_num[fr] == train_num[fc]:
                    continue
                if fil_lens[fr] == fil_lens[fc] and pr_s == pc_s:
                    continue
                dist = pc_s - pr_e - 1
                if dist < 0:
                    over[-dist - 1, fc, fr] += 1
                elif 0 < dist <= CmFm1:
                    non_over[dist - 1, fc, fr] += 1
                else:
                    next_to[fc, fr] += 1
    return over.astype(np.int32), non_over.astype(np.int32), next_to.astype(np.int32)


def pair_msas(over, start_pos, fil_lens, train_num, uinds, codes, data,
              count_threshold: int, filter_size: int):
    """src/SEARCH/extractions.jl:18-114 (get_f_pair_starts :116-137, get_span_len
    :139-147, msa_fill :149-181, msa_pseudocount :183-190), in FP64.
    codes: (T, N, M, C) float (Julia (T, C, M, N)).  Returns (pairs list of
    (fr, fc, o_len) 1-based, span_len int array, pfms list of (4, span) arrays)."""
    maxlen_o, K, _ = over.shape
    N, _, C = start_pos.shape
    max_span = 2 * filter_size - 1
    # findall on Julia (K, K, maxlen): fr fastest, then fc, then o_len
    pairs = []
    for o in range(maxlen_o):
        for fc in range(K):
            for fr in range(K):
                if over[o, fc, fr] > count_threshold:
                    pairs.append((fr + 1, fc + 1, o + 1))
    onehot = data.astype(np.float64)
    spans, pfms = [], []
    for (fr, fc, o_len) in pairs:
        fl1 = int(fil_lens[fr - 1]); fl2 = int(fil_lens[fc - 1])
        span = o_len if o_len >= fl2 else fl1 - o_len + fl2
        t1 = int(train_num[fr - 1]) - 1; t2 = int(train_num[fc - 1]) - 1
        f1 = int(uinds[fr - 1]) - 1; f2 = int(uinds[fc - 1]) - 1
        msa = np.zeros(4 * max_span)
        for n in range(N):
            starts = np.zeros(C, bool)
            for c in range(1, C + 1):
                f1_at = o_len + c - fl1
                if start_pos[n, fc - 1, c - 1] and f1_at > 0 and start_pos[n, fr - 1, f1_at - 1]:
                    starts[f1_at - 1] = True
            for c in range(1, C - span + 2):
                if not starts[c - 1]:
                    continue
                off = (c - 1) * 4
                f2_start = c + fl1 - o_len
                avg = (codes[t1, n, f1, c - 1] + codes[t2, n, f2, f2_start - 1]) / 2
                msa[: 4 * span] += avg * onehot[n, off: off + 4 * span]
        msa[: 4 * span] += 0.1
        m3 = msa.reshape(max_span, 4).T        # (4, max_span)
        pfm = m3 / np.sum(m3[:, 0])
        spans.append(span)
        pfms.append(pfm[:, :span])
    return pairs, np.asarray(spans, np.int32), pfms


# ----------------------------------------------------------------------------------
# a23: save_pfms_as_transfac (src/SAVE/save_learned_results.jl:184-217)
# ----------------------------------------------------------------------------------
def julia_float32_string(x) -> str:
    """Julia ``string(::Float32)``: the shortest decimal digits that read back to the
    same Float32 (numpy's Dragon4 in ``unique`` mode), written positionally when the
    decimal point position pt (value = 0.d1d2.. x 10^pt) satisfies -4 < pt <= 6
    (integral values get a trailing ``.0``), else as ``d.ddde<exp>`` (``1.0e-5``).
    Transfac values (pfm * 1000, in (0, 1000]) are always positional."""
    x = np.float32(x)
    if np.isnan(x):
        return "NaN"
    if np.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if x == 0:
        return "-0.0" if np.signbit(x) else "0.0"
    sign = "-" if x < 0 else ""
    s = np.format_float_scientific(abs(x), unique=True, trim='-', exp_digits=1)
    mant, exp = s.split('e')
    digits = mant.replace('.', '').rstrip('0') or '0'
    pt = int(exp) + 1
    k = len(digits)
    if -4 < pt <= 6:
        if pt <= 0:
            out = "0." + "0" * (-pt) + digits
        elif pt < k:
            out = digits[:pt] + "." + digits[pt:]
        else:
            out = digits + "0" * (pt - k) + ".0"
    else:
        out = digits[0] + "." + (digits[1:] or "0") + "e" + str(pt - 1)
    return sign + out


def transfac_text(pfm_4w) -> str:
    """One transfac file body as written by save_pfms_as_transfac (:186-196)."""
    q = (np.asarray(pfm_4w, dtype=f32) * f32(1000)).astype(f32)
    lines = ["ID\t", "XX\t", "BF\t", "XX\t", "P0\tA\tC\tG\tT"]
    for j in range(1, q.shape[1] + 1):
        row = ("0" + str(j)) if j < 10 else str(j)
        vals = "\t".join(julia_float32_string(q[a, j - 1]) for a in range(4))
        lines.append(row + "\t" + vals)
    lines.append("XX\t")
    return "\n".join(lines) + "\n"
