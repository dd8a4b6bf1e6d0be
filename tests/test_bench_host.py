"""Host-side pieces of bench.py (no GPU): the padded FFT lengths it reports
are the library's rule, the FP64 work counts follow the reference's
operations, and every name the script loads is defined -- its GPU paths run
only on a GPU machine, so a misspelt name there would otherwise first show as a
failed benchmark."""
import ast
import builtins
import math
import os

import pytest

from conftest import REPO

bench = pytest.importorskip("bench")


@pytest.mark.parametrize("n,L", [(4, 8), (5, 12), (7, 16), (15, 32), (24, 48), (48, 96), (63, 128), (64, 128),
                                 (96, 192), (128, 256), (192, 384), (256, 512), (257, 0)])
def test_padded_length_is_the_librarys_rule(n, L):
    # the smallest 2^k or 3 * 2^k in 8 .. 512 holding 2n - 1 points (choose_fft_length in the library)
    assert bench.padded_length(n) == L


def test_fp64_work_counts():
    w = bench.fp64_work_per_kick([63, 63, 63])
    M = 128 ** 3
    assert w["padded_grid"] == [128, 128, 128]
    assert w["fft_flops_reference_count"] == 3 * 5 * M * math.log2(M)
    assert w["igf_transcendentals"] == 7 * 64 ** 3


def test_every_name_bench_loads_is_defined():
    tree = ast.parse(open(os.path.join(REPO, "bench.py")).read())
    defined = set(dir(builtins)) | {"__file__"}
    for node in ast.walk(tree):
        if isinstance(node, (ast.FunctionDef, ast.ClassDef)):
            defined.add(node.name)
        elif isinstance(node, ast.Import):
            defined.update((a.asname or a.name).split(".")[0] for a in node.names)
        elif isinstance(node, ast.ImportFrom):
            defined.update(a.asname or a.name for a in node.names)
        elif isinstance(node, ast.Name) and isinstance(node.ctx, (ast.Store, ast.Del)):
            defined.add(node.id)
        elif isinstance(node, ast.arg):
            defined.add(node.arg)
        elif isinstance(node, ast.ExceptHandler) and node.name:
            defined.add(node.name)
    loads = {n.id for n in ast.walk(tree) if isinstance(n, ast.Name) and isinstance(n.ctx, ast.Load)}
    assert not loads - defined
