"""Generators are deterministic and portable; the text format round-trips."""
from __future__ import annotations

import numpy as np

import sbclip_gen as gen
from conftest import digest


def test_sincos_accuracy():
    t = np.linspace(0.0, 2 * np.pi, 20001)
    s, c = gen.sincos(t)
    assert np.abs(s - np.sin(t)).max() < 1e-15
    assert np.abs(c - np.cos(t)).max() < 1e-15


def test_star_is_ccw_and_deterministic():
    a = gen.star(500, 3)
    b = gen.star(500, 3)
    assert np.array_equal(a, b)
    area = 0.5 * np.sum(a[:, 0] * np.roll(a[:, 1], -1) - np.roll(a[:, 0], -1) * a[:, 1])
    assert area > 0


def test_pinned_inputs(digests):
    b, c = gen.pair_small()
    assert digest(b, c) == digests["pair_10k_8k"]["input_sha256"]


def test_text_round_trip(tmp_path):
    xy = gen.star(100, 5)
    p = tmp_path / "p.txt"
    gen.write_poly(p, xy)
    assert np.array_equal(gen.read_poly(p), xy)
    gen.write_poly(p, xy, sep=" ")
    assert np.array_equal(gen.read_poly(p), xy)
