"""The register-FFT transform lengths are listed in three places that must agree: the
multi-iteration X-step's instantiations (csrc/xiter_v*.cu), the streaming D-step
transforms' (csrc/dstream_v*.cu), and the padding table of the training server
(csrc/server.cpp's friendly_L) with its Python mirror (serve.REGISTER_LG).  Read from
the sources, no GPU needed."""
import glob
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cdlmotif.jl_gb300", "csrc")


def _lengths(pattern, macro):
    out = set()
    for path in glob.glob(os.path.join(CSRC, pattern)):
        for n1, p in re.findall(macro + r"\((\d+),\s*(\d+)", open(path).read()):
            out.add(int(n1) * int(p))
    return out


def test_xstep_and_dstep_lengths_agree():
    xs = _lengths("xiter_v*.cu", "XITER_VARIANT")
    ds = _lengths("dstream_v*.cu", "DSTREAM_VARIANT")
    assert xs and xs == ds


def test_server_padding_table_matches_the_kernels(pkg):
    from cdlmotif_gb300 import serve
    src = open(os.path.join(CSRC, "server.cpp")).read()
    table = re.search(r"kRegLg\[\]\s*=\s*\{([^}]*)\}", src).group(1)
    cpp = [int(v) for v in re.findall(r"\d+", table)]
    assert cpp == sorted(cpp) and tuple(cpp) == tuple(serve.REGISTER_LG)
    assert set(cpp) <= _lengths("xiter_v*.cu", "XITER_VARIANT")


def test_per_lane_tables_cover_every_variant():
    """Every per-lane DFT length P of a variant has its cos/sin table (toff(P) >= 0) and
    the tables do not overlap."""
    src = open(os.path.join(CSRC, "regfft.cuh")).read()
    ps = [int(v) for v in re.search(r"kPrimesW\[\]\s*=\s*\{([^}]*)\}", src).group(1).split(",")]
    offs = {int(p): int(o) for p, o in re.findall(r"p == (\d+) \? (\d+)", src)}
    assert sorted(offs) == sorted(ps)
    o = 0
    for p in ps:
        assert offs[p] == o, p
        o += p
    n_tab = re.search(r"constexpr int kTrigW = ([^;]*);", src).group(1)
    assert eval(n_tab.replace("\n", " ")) == o
    used = set()
    for path in glob.glob(os.path.join(CSRC, "xiter_v*.cu")) + glob.glob(os.path.join(CSRC, "dstream_v*.cu")):
        used |= {int(p) for _, p in re.findall(r"VARIANT\((\d+),\s*(\d+)", open(path).read())}
    assert used <= set(ps)


def test_friendly_padding_reaches_a_register_length_up_to_992(pkg):
    """With the server's 8 % rule every transform length from 300 to 992 (W = 16: L from
    43 to 216) pads to a register-FFT length."""
    from cdlmotif_gb300 import serve
    reg = set(serve.REGISTER_LG)
    for L in range(43, 217):
        Lp = serve.friendly_length(L, 16)
        assert 4 * Lp + 128 in reg, L
    assert np.all(np.diff(serve.REGISTER_LG) > 0)
