"""FASTA ingest on the GPU (cdlgb_load_fasta) against the oracle's restatement of
read_fasta + data_2_dummy (src/LOAD/read.jl:2-28, src/LOAD/to_dummy.jl:27-38): the
loaded one-hot matrix is identical, and errors are reported."""
import numpy as np
import pytest

from oracle import search_oracle as SO

from test_oracle_cpu import FASTA_TEXT

pytestmark = pytest.mark.gpu


def _ctx(pkg):
    return pkg.CDL(pkg.CDLSetup(M=2, filter_size=2))


@pytest.mark.parametrize("max_entries", [10000, 2])
def test_load_fasta_small(pkg, built_lib, max_entries):
    ref, reads = SO.read_fasta_onehot(FASTA_TEXT, max_entries)
    with _ctx(pkg) as c:
        info = c.load_fasta(FASTA_TEXT, max_entries)
        assert info["N"] == len(reads) and info["L"] == 6
        assert info["wrong_length"] == (1 if max_entries > 2 else 0)
        np.testing.assert_array_equal(c.data(), ref)


def test_load_fasta_random_and_scan(pkg, built_lib, tmp_path):
    rng = np.random.default_rng(3)
    N, L = 700, 150
    bases = rng.integers(0, 4, (N, L))
    lines = []
    for n in range(N):
        seq = "".join("acgt"[b] if (n + i) % 7 == 0 else "ACGT"[b] for i, b in enumerate(bases[n]))
        if n % 50 == 3:
            seq = seq[:40] + "N" + seq[41:]          # dropped
        lines.append(f">read{n} x\n" + "\n".join(seq[i:i + 60] for i in range(0, L, 60)))
    text = ("\n".join(lines) + "\n").encode()
    path = tmp_path / "reads.fa"
    path.write_bytes(text)
    ref, reads = SO.read_fasta_onehot(text)
    with _ctx(pkg) as c, _ctx(pkg) as c2:
        info = c.load_fasta(str(path))
        assert info["N"] == len(reads) == N - 14 and info["L"] == L
        np.testing.assert_array_equal(c.data(), ref)
        # the scans see the same data as through load_data
        c2.load_data(ref)
        pwms = [np.log2((rng.dirichlet(np.ones(4), 8).T + 0.05) / 0.45).astype(np.float32)]
        th = np.array([2.0], np.float32)
        np.testing.assert_array_equal(pkg.overlapping_scan(c, pwms, th)[0],
                                      pkg.overlapping_scan(c2, pwms, th)[0])


def test_load_fasta_errors(pkg, built_lib):
    with _ctx(pkg) as c:
        with pytest.raises(pkg.CDLGBError) as e:
            c.load_fasta(b">a\nACGR\n")               # not ACGT: the reference's KeyError
        assert e.value.status == -1
        with pytest.raises(pkg.CDLGBError):
            c.load_fasta(b">a\nACGN\n>b\nNNNN\n")     # every record dropped
