"""Restart-vector files in the reference's wf_self_as_guess.out format, host side
(no GPU): the writer of src/minres.cpp:59-70 (length line, then "key amplitude"
with the amplitude at 12 significant digits) and the reader readPsi of
src/main.cpp:288-307."""
import os

import numpy as np
import pytest

import sfci_gb300 as sg


def expected_text(keys, amps):
    # the reference streams `basis[i] << ' ' << setprecision(12) << amp[i]`:
    # default float format with 12 significant digits, i.e. printf's %.12g
    return "%d\n" % len(amps) + "".join("%d %s\n" % (int(k), "%.12g" % a) for k, a in zip(keys, amps))


def test_write_matches_reference_format(tmp_path):
    rng = np.random.default_rng(2)
    keys = np.sort(rng.choice(1 << 40, 500, replace=False)).astype(np.uint64)
    amps = rng.normal(size=500) * np.exp2(rng.uniform(-40, 10, 500))
    amps[:3] = [0.5, -1e-05, 123456789.123456789]
    p = tmp_path / "wf_self_as_guess.out"
    sg.psi_write(str(p), keys, amps)
    assert p.read_text() == expected_text(keys, amps)


def test_read_round_trip_and_whitespace(tmp_path):
    rng = np.random.default_rng(3)
    keys = np.sort(rng.choice(1 << 56, 300, replace=False)).astype(np.uint64)
    amps = rng.normal(size=300)
    p = tmp_path / "wf"
    sg.psi_write(str(p), keys, amps)
    k, a = sg.psi_read(str(p), 56)
    assert np.array_equal(k, keys)
    assert np.array_equal(a, np.array([float("%.12g" % x) for x in amps]))
    # readPsi uses fscanf, so any whitespace separates fields
    p2 = tmp_path / "wf2"
    p2.write_text("2\n\n  7   0.25\t\n9\n-1.5e-3\n")
    k, a = sg.psi_read(str(p2), 56)
    assert list(k) == [7, 9] and list(a) == [0.25, -1.5e-3]
    sg.psi_write(str(p), np.zeros(0, np.uint64), np.zeros(0))
    assert p.read_text() == "0\n"
    assert sg.psi_read(str(p), 56)[0].size == 0


def test_two_word_keys(tmp_path):
    lo = np.array([5, 0, 2**63 + 1], np.uint64)
    hi = np.array([0, 1, 2**3], np.uint64)
    keys = np.stack([lo, hi], axis=1)
    amps = np.array([1.0, -2.0, 3.5])
    p = tmp_path / "wf128"
    sg.psi_write(str(p), keys, amps, key_words=2)
    want = [int(l) + (int(h) << 64) for l, h in zip(lo, hi)]
    assert p.read_text() == expected_text(want, amps)
    k, a = sg.psi_read(str(p), 70, key_words=2)
    assert np.array_equal(k, keys) and np.array_equal(a, amps)


def test_read_errors(tmp_path):
    p = tmp_path / "bad"
    p.write_text("1\n%d 0.5\n" % (1 << 20))
    with pytest.raises(sg.SfciError) as e:
        sg.psi_read(str(p), 20)  # bit 20 is beyond 20 spin orbitals
    assert e.value.status == "SFCI_ERR_ARG"
    for text in ("3\n1 0.5\n2 0.25\n", "1\n1 x\n", "1\n-1 0.5\n", "abc\n"):
        p.write_text(text)
        with pytest.raises(sg.SfciError) as e:
            sg.psi_read(str(p), 20)
        assert e.value.status == "SFCI_ERR_IO", text
    with pytest.raises(sg.SfciError) as e:
        sg.psi_read(str(tmp_path / "missing"), 20)
    assert e.value.status == "SFCI_ERR_IO"
