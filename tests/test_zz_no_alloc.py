"""sfci_dot_noalloc: the dot product for callers that cannot allocate device memory.

Some callers run inside another framework's device-memory pool, where the
framework has reserved the GPU up front. Others are hosts whose hot loop must
not allocate. For both, a cudaMalloc either fails or is not allowed. The entry
point keeps its scratch in a fixed device array, and the caller passes inputs
and the output in its own device memory. This test calls it through the C ABI
twice in a row. Both results must match sfci_dot on the same data within the
1e-12 relative tolerance the other scalar tests use. The file is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from parity import close

import sfci_gb300 as sg

pytestmark = pytest.mark.gpu


def _lib():
    L = sg.load_library()
    f = L.sfci_dot_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p,
                  C.c_void_p]
    return L


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint64:
        a = a.view(np.int64)
    return torch.from_numpy(a.copy()).to("cuda")


def _check(golden_in, torch, xk, xa, yk, ya, words, path, norb, ne):
    L = _lib()
    c = sg.Context(path, norb, ne, Nd=200000)
    ref = c.vec_from(xk, xa).dot(c.vec_from(yk, ya))
    dxk, dxa, dyk, dya = _dev(torch, xk), _dev(torch, xa), _dev(torch, yk), _dev(torch, ya)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(float("nan"))
        st = L.sfci_dot_noalloc(dxk.data_ptr(), dxa.data_ptr(), len(xa), dyk.data_ptr(), dya.data_ptr(), len(ya),
                                words, out.data_ptr(), stream)
        assert st == 0, L.sfci_last_error()
        torch.cuda.synchronize()
        assert close(float(out.item()), ref), (float(out.item()), ref)


def test_dot_noalloc_matches_dot(golden_in):
    torch = pytest.importorskip("torch")
    g, path = golden_in("c1")
    _check(golden_in, torch, g["B_in_keys"], g["B_in_amps"], g["B_keys"], g["B_amps"], 1, path, 20, 10)


def test_dot_noalloc_two_word_keys(golden_in):
    torch = pytest.importorskip("torch")
    g, path = golden_in("c1")
    # the same vectors with every key in its two-word form (high word 0) and an
    # extra high bit on a third of the keys, so both words take part in the order
    def wide(k, salt):
        w = np.zeros((len(k), 2), np.uint64)
        w[:, 0] = k
        w[::3, 1] = salt
        order = np.lexsort((w[:, 0], w[:, 1]))
        return w[order], order
    xk, ox = wide(g["B_in_keys"], 1)
    yk, oy = wide(g["B_keys"], 1)
    L = _lib()
    dxk, dxa = _dev(torch, xk), _dev(torch, g["B_in_amps"][ox])
    dyk, dya = _dev(torch, yk), _dev(torch, g["B_amps"][oy])
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    xi = {(int(a), int(b)): v for (a, b), v in zip(xk, g["B_in_amps"][ox])}
    ref = sum(v * xi.get((int(a), int(b)), 0.0) for (a, b), v in zip(yk, g["B_amps"][oy]))
    for _ in range(2):
        st = L.sfci_dot_noalloc(dxk.data_ptr(), dxa.data_ptr(), len(xk), dyk.data_ptr(), dya.data_ptr(), len(yk), 2,
                                out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert st == 0, L.sfci_last_error()
        torch.cuda.synchronize()
        assert close(float(out.item()), ref)


def test_dot_noalloc_leaves_free_memory_unchanged(golden_in):
    """After the first call (which looks up the fixed array's address), repeated
    calls, including ones near the size limit, change the device's free memory
    by nothing: the entry point allocates no device memory of its own."""
    torch = pytest.importorskip("torch")
    g, _ = golden_in("c1")
    L = _lib()
    n = (1 << 23) - 7  # two vectors of this length: close to the 16,777,216-entry limit
    big_k = torch.arange(0, 2 * n, 2, dtype=torch.int64, device="cuda")
    big_a = torch.ones(n, dtype=torch.float64, device="cuda")
    dxk, dxa = _dev(torch, g["B_in_keys"]), _dev(torch, g["B_in_amps"])
    dyk, dya = _dev(torch, g["B_keys"]), _dev(torch, g["B_amps"])
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call(xk, xa, nx, yk, ya, ny):
        st = L.sfci_dot_noalloc(xk.data_ptr(), xa.data_ptr(), nx, yk.data_ptr(), ya.data_ptr(), ny, 1,
                                out.data_ptr(), stream)
        assert st == 0, L.sfci_last_error()

    call(dxk, dxa, len(g["B_in_amps"]), dyk, dya, len(g["B_amps"]))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        call(dxk, dxa, len(g["B_in_amps"]), dyk, dya, len(g["B_amps"]))
        call(big_k, big_a, n, big_k, big_a, n)
    torch.cuda.synchronize()
    assert float(out.item()) == float(n)
    assert torch.cuda.mem_get_info()[0] == free0
