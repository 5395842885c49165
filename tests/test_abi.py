"""The C-ABI library loads, exports every symbol include/pmcg.h declares, and
its host-side entry points behave (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pmcg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#.*", "", src)
    names = set()
    for stmt in src.split(";"):
        stmt = " ".join(stmt.split())
        if "typedef" in stmt or "{" in stmt or "}" in stmt:
            stmt = stmt.split("}")[-1]
            if "typedef" in stmt:
                continue
        m = re.match(r"^[\w\s\*]*?\b(\w+)\s*\(", stmt)
        if m and m.group(1) not in ("if", "return"):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(pmcg):
    L = pmcg.load()
    names = declared_functions()
    assert len(names) > 50
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_signature_table_covers_header(pmcg):
    table = {s[0] for s in pmcg.SIGNATURES}
    assert set(declared_functions()) <= table


def test_error_chain(pmcg):
    L = pmcg.load()
    e = L.addError(-9008, b"first", None, 1)
    e2 = L.addError(-9002, b"second", e, 2)
    assert L.isError(e2) == 1 and L.getErrorValue(e2) == -9002
    assert e2.contents.next.contents.errValue == -9008
    p = C.POINTER(pmcg.Error)(e2.contents)
    L.purgeError(C.byref(p))
    assert not p


def test_tempering_matches_reference_formula(pmcg):
    assert pmcg.get_tempering_beta(0, 3, 0.1, 10) == 1.0
    assert pmcg.get_tempering_beta(1, 9, 0.1, 10) == 1.0
    assert abs(pmcg.get_tempering_beta(1, 4, 0.1, 10) - (4 / 8 * 0.9 + 0.1)) < 1e-15
    assert abs(pmcg.get_tempering_beta(2, 4, 0.01, 10) - np.exp(4 / 8 * -np.log(0.01) + np.log(0.01))) < 1e-15
    with pytest.raises(pmcg.PmcgError):
        pmcg.get_tempering_beta(2, 1, 0.0, 10)
    with pytest.raises(pmcg.PmcgError):
        pmcg.get_tempering_beta(7, 1, 0.1, 10)


def test_mixture_alloc_cholesky_and_text_roundtrip(pmcg, tmp_path):
    rng = np.random.default_rng(0)
    K, D = 3, 4
    A = rng.normal(size=(K, D, D))
    cov = np.einsum("kij,klj->kil", A, A) + np.eye(D)
    mu = rng.normal(size=(K, D))
    m = pmcg.MixMvdens.from_arrays([0.2, 0.3, 0.5], mu, cov=cov, df=3).cholesky()
    w, mu2, L = m.arrays()
    np.testing.assert_allclose(np.einsum("kij,klj->kil", L, L), cov, rtol=1e-12)
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    path = str(tmp_path / "proposal").encode()
    f = libc.fopen(path, b"w")
    pmcg.load().mix_mvdens_dump(f, m.p)
    libc.fclose(f)
    f = libc.fopen(path, b"r")
    p2 = pmcg.call("mix_mvdens_dwnp", f)
    libc.fclose(f)
    m2 = pmcg.MixMvdens.__new__(pmcg.MixMvdens)
    m2.p, m2.K, m2.D = p2, K, D
    w3, mu3, L3 = m2.arrays()
    np.testing.assert_allclose(w3, w, rtol=1e-15)
    np.testing.assert_allclose(mu3, mu, rtol=1e-15)
    np.testing.assert_allclose(np.einsum("kij,klj->kil", L3, L3), cov, rtol=1e-12)
    assert m2.df == 3
    assert abs(pmcg.effective_number_of_components(m) - 1 / np.sum(np.square([0.2, 0.3, 0.5]))) < 1e-14


def test_non_pd_covariance_is_rejected(pmcg):
    m = pmcg.MixMvdens.from_arrays([1.0], [[0.0, 0.0]], cov=[[[1.0, 2.0], [2.0, 1.0]]])
    with pytest.raises(pmcg.PmcgError) as e:
        m.cholesky()
    assert e.value.code == -9003


def test_parabox_and_simu_containers(pmcg):
    pb = pmcg.Parabox([0, -1], [1, 1])
    L = pmcg.load()
    x = (C.c_double * 2)(0.5, 0.0)
    assert L.isinBox(pb.p, x) == 1
    x = (C.c_double * 2)(1.5, 0.0)
    assert L.isinBox(pb.p, x) == 0
    with pytest.raises(pmcg.PmcgError):
        pmcg.call("add_slab", pb.p, 0, 1.0, 0.0)
    ps = pmcg.PmcSimu(100, 3)
    assert ps.X.shape == (100, 3) and ps.weights.shape == (100,)
    pmcg.call("pmc_simu_realloc", ps.p, 250)
    assert ps.X.shape == (250, 3)


def test_device_calls_fail_cleanly_without_gpu(pmcg):
    if pmcg.device_count() > 0:
        pytest.skip("a GPU is present")
    m = pmcg.MixMvdens.from_arrays([1.0], [[0.0, 0.0]], cov=[np.eye(2)])
    with pytest.raises(pmcg.PmcgError) as e:
        pmcg.mix_log_pdf_batch(m, np.zeros((4, 2)))
    assert e.value.code == -9001


def test_weight_step_rejects_host_callbacks(pmcg):
    """Only the device posterior is accepted by the weight step."""
    L = pmcg.load()
    ps = pmcg.PmcSimu(10, 2)
    m = pmcg.MixMvdens.from_arrays([1.0], [[0.0, 0.0]], cov=[np.eye(2)])
    cb = pmcg.LOGPDF_FN(lambda extra, x, err: 0.0)
    q = C.cast(L.mix_mvdens_log_pdf_void, C.c_void_p)
    with pytest.raises(pmcg.PmcgError) as e:
        pmcg.call("generic_get_importance_weight_and_deduced_verb", ps.p, m.p, q, C.cast(cb, C.c_void_p), None,
                  None, 1.0, 1)
    assert e.value.code == -9006


def test_server_and_batch_need_a_gpu(pmcg):
    if pmcg.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(pmcg.PmcgError) as e:
        pmcg.Server()
    assert e.value.code == -9001
    with pytest.raises(pmcg.PmcgError):
        pmcg.call("pmcg_batch_create", 0, None)


def test_sample_file_roundtrip(pmcg, tmp_path):
    """out_pmc_simu_cosmo_pmc / pmc_simu_from_file (exec/exec_helper.c:351-427 layout):
    counted rows only, unnormalised log-weight back from the normalised weights."""
    rng = np.random.default_rng(3)
    N, D = 50, 4
    ps = pmcg.PmcSimu(N, D)
    X = rng.normal(size=(N, D))
    logw = rng.normal(size=N) * 3
    flg = np.ones(N, dtype=np.int16)
    flg[[3, 17]] = 0
    ps.X[:] = X
    ps.flg[:] = flg
    ps.indices[:] = rng.integers(0, 7, N)
    mx = logw[flg == 1].max()
    ls = mx + np.log(np.sum(np.exp(logw[flg == 1] - mx)))
    ps.weights[:] = np.exp(logw - ls)        # normalised, as after normalize_importance_weight
    ps.s.isLog = 0
    ps.s.logSum = ls
    path = tmp_path / "pmcsim"
    ps.write(path, [f"p{i}" for i in range(D)])
    text = path.read_text().splitlines()
    assert text[0] == "# npar = 4, n_ded = 0" and len([t for t in text if not t.startswith("#")]) == N - 2
    back = pmcg.PmcSimu.read(path, 1000, D)
    keep = flg == 1
    assert back.N == N - 2 and back.s.isLog == 0
    np.testing.assert_allclose(back.X, X[keep], rtol=1e-8, atol=1e-8)
    np.testing.assert_array_equal(back.indices, ps.indices[keep])
    np.testing.assert_allclose(back.s.logSum, ls, rtol=1e-8)
    np.testing.assert_allclose(back.weights, np.exp(logw[keep] - ls), rtol=1e-7)
    assert np.all(back.flg == 1)
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    f = libc.fopen(str(path).encode(), b"r")
    with pytest.raises(pmcg.PmcgError):
        pmcg.call("pmc_simu_from_file", f, 100, D, 0, None, -1)  # nclipw < 0
    libc.fclose(f)


def test_c_caller_compiles_against_the_header(pmcg, tmp_path):
    """tests/c/dropin_sequence.c, a C caller of the pmclib-named entry points,
    compiles with gcc against include/pmcg.h and links to libpmcg.so (it runs
    under -m gpu)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    lib_dir = os.path.join(ROOT, "cosmopmc_gb300")
    out = tmp_path / "dropin_sequence"
    r = subprocess.run([gcc, "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "c", "dropin_sequence.c"), "-L", lib_dir, "-lpmcg",
                        f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.exists()
