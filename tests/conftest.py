import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def kat():
    """Known-answer data of the reference's scripts/log (see tests/golden/make_golden.py)."""
    return dict(np.load(os.path.join(GOLDEN, "lambda_kat.npz")))


@pytest.fixture(scope="session")
def score_logs():
    return dict(np.load(os.path.join(GOLDEN, "score_logs.npz")))


@pytest.fixture(scope="session")
def built_lib():
    """libdtwx.so built in-tree (nvcc cross-compiles without a GPU)."""
    from dtwax_gb300 import build
    build.build()
    import dtwax_gb300
    return dtwax_gb300.load_library()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def write_kat_files(kat, folder):
    """Write the lambda FASTA and k-mer model of the golden fixture as files."""
    fasta = os.path.join(folder, "reference.fasta")
    model = os.path.join(folder, "dna_kmer_model.txt")
    seq = kat["seq"].tobytes().decode()
    with open(fasta, "w") as f:
        f.write(str(kat["fasta_header"]) + "\n")
        for i in range(0, len(seq), 60):
            f.write(seq[i:i + 60] + "\n")
    with open(model, "w") as f:
        for code in range(4096):
            k = "".join("ACGT"[(code >> (2 * (5 - j))) & 3] for j in range(6))
            f.write(f"{k} {kat['model_means'][code]:.6f} {kat['model_stdevs'][code]:.6f}\n")
    return fasta, model
