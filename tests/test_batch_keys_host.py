"""The check of keys uploaded into a batched context (first_bad_batched_key in
csrc/gen.cuh, called by sfci_vec_upload), compiled for the host.

A batched context's kernels pick each key's Hamiltonian by the instance tag in
bits 123..127, so an upload must reject a tag that names no instance and a key
with a bit at or above its instance's spin-orbital count.  The check is
compared with a Python model on random keys of instances below, at and above
64 spin orbitals, with the edge bits set one at a time."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "sfci_gb300", "csrc")
SHIFT = 59


@pytest.fixture(scope="module")
def bk(tmp_path_factory):
    d = tmp_path_factory.mktemp("bk")
    so = str(d / "gen_host.so")
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + CSRC, "-I/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "native", "gen_host.cpp"), os.path.join(CSRC, "ham.cpp"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = C.CDLL(so)
    L.gh_first_bad_batched_key.restype = C.c_ulonglong
    L.gh_first_bad_batched_key.argtypes = [np.ctypeslib.ndpointer(np.uint64), C.c_ulonglong,
                                           np.ctypeslib.ndpointer(np.int32), C.c_int]
    return L


def first_bad(L, keys, inst_N):
    kw = np.ascontiguousarray(np.asarray(keys, np.uint64).reshape(-1, 2))
    n = np.ascontiguousarray(inst_N, np.int32)
    return L.gh_first_bad_batched_key(kw.reshape(-1) if kw.size else np.zeros(2, np.uint64), len(kw), n, len(n))


def model_ok(key, inst_N):
    tag = key >> 123
    return tag < len(inst_N) and (key & ((1 << 123) - 1)) >> inst_N[tag] == 0


def words(key):
    return [key & (2 ** 64 - 1), key >> 64]


INST_N = [8, 64, 120, 100]


def test_valid_keys_pass(bk):
    rng = np.random.default_rng(3)
    keys = []
    for t, N in enumerate(INST_N):
        for _ in range(200):
            body = int.from_bytes(rng.bytes(16), "little") & ((1 << N) - 1)
            keys.append(words(body | (t << 123)))
    assert first_bad(bk, keys, INST_N) == len(keys)
    assert first_bad(bk, np.zeros((0, 2), np.uint64), INST_N) == 0


@pytest.mark.parametrize("t,N", list(enumerate(INST_N)))
def test_edge_bits(bk, t, N):
    for b in range(max(0, N - 3), 123):
        key = (1 << b) | (t << 123)
        want_ok = model_ok(key, INST_N)
        assert want_ok == (b < N)
        got = first_bad(bk, [words(1 | (t << 123)), words(key)], INST_N)
        assert got == (2 if want_ok else 1), (t, N, b)


def test_tags_beyond_the_batch(bk):
    for ninst in (1, 4, 31, 32):
        inst_N = [64] * ninst
        for tag in range(32):
            got = first_bad(bk, [words(tag << 123)], inst_N)
            assert got == (1 if tag < ninst else 0), (ninst, tag)


def test_random_keys_against_model(bk):
    rng = np.random.default_rng(11)
    for _ in range(300):
        key = int.from_bytes(rng.bytes(16), "little")
        # mostly valid keys, with a random bit or tag spoiled now and then
        t = int(rng.integers(0, 5))
        N = INST_N[t] if t < len(INST_N) else 64
        key = (key & ((1 << N) - 1)) | (t << 123)
        if rng.random() < 0.3:
            key |= 1 << int(rng.integers(0, 123))
        got = first_bad(bk, [words(key)], INST_N)
        assert got == (1 if model_ok(key, INST_N) else 0), hex(key)
