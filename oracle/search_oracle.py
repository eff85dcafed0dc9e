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
