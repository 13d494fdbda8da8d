"""CPU-side checks of the product library: it builds for sm_103a, loads, exports every
entry point include/inspire_gb300.h declares, encodes responses byte-identically to the
oracle, and refuses to run without a GPU (no CPU fallback)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_package

HEADER = os.path.join(ROOT, "include", "inspire_gb300.h")


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void\*?|uint64_t)\s+\*?(ig_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg._build.build())
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_library_targets_sm_103a(pkg):
    assert "arch=compute_103a,code=sm_103a" in " ".join(pkg._build.ARCH)


def test_response_wire_matches_oracle(pkg, oracle):
    d = np.load(os.path.join(ROOT, "tests", "golden", "d256_respond.npz"))
    P = oracle.Params(n=int(d["n"]), q=int(d["q"]), p=int(d["p"]), sigma=float(d["sigma"]))
    cache = oracle.Cache(P, int(d["gamma"]), d["w_seed"].tobytes())
    a, b = cache.respond_per_query(d["columns"], d["query_a"], d["query_b"], d["y_body"])
    resp = pkg.ServerResponse(a, b, int(d["gamma"]), P.q).to_binary()
    assert resp == oracle.response_bytes(a, b, int(d["gamma"]), P.q)
    assert oracle.fnv1a(resp) == int(d["golden_fnv"])
    # 36-bit switched wire: 10,446 bytes at gamma 256, d 2048.
    n = 2048
    ms = pkg.MOD_SWITCH_TARGET_36BIT
    a2 = (np.arange(n, dtype=np.uint64) * 977) % ms
    b2 = (np.arange(n, dtype=np.uint64) * 31) % ms
    w = pkg.ServerResponse(a2, b2, 256, ms).to_binary()
    assert len(w) == 10_446 and w == oracle.response_bytes(a2, b2, 256, ms)


def test_non_canonical_coefficient_is_refused(pkg):
    a = np.full(256, pkg.DEFAULT_Q, dtype=np.uint64)
    with pytest.raises(pkg.PirError):
        pkg.ServerResponse(a, a, 16).to_binary()


def test_no_cpu_fallback_without_gpu(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.PirError, match="no CPU fallback"):
        pkg.Context(0)


def test_mod_switch_noise_gate(pkg):
    p = pkg.InspireParams.d2048()
    pkg.check_mod_switch_noise_budget(p, pkg.MOD_SWITCH_TARGET_36BIT)
    with pytest.raises(pkg.PirError):
        pkg.check_mod_switch_noise_budget(p, 12289)
