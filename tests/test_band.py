"""The band program's k-point path (makePathKPoints,
src/olcao/kpoints.f90:313-534), on known answers: host logic, no GPU."""

import math

import numpy as np
import pytest

from olcao_gb300 import band


def _cubic(a=1.0):
    return a * np.eye(3)            # columns a, b, c: reciprocal vectors 2 pi / a


def test_reciprocal_vectors_and_fractional_round_trip():
    rv = np.array([[4.0, 0.3, 0.1], [0.2, 5.0, 0.4], [0.0, 0.5, 6.0]])
    B = band.recip_vectors(rv)
    assert np.allclose(B @ rv, 2.0 * math.pi * np.eye(3))
    f = np.array([[0.1, -0.2, 0.3], [0.5, 0.5, 0.0]])
    assert np.allclose(band.to_fractional(rv, f @ B), f)


def test_path_of_only_high_symmetry_points():
    paths = [np.array([[0, 0, 0], [0.5, 0, 0], [0.5, 0.5, 0]])]
    k, mag, w, idx = band.path_kpoints(_cubic(), paths, 3)
    assert np.allclose(k, paths[0] * 2.0 * math.pi)
    assert np.allclose(mag, [0.0, math.pi, 2.0 * math.pi])
    assert np.allclose(w, 2.0 / 3) and idx == [1, 2, 3]


def test_interpolated_path_counts_steps_as_the_reference():
    # Gamma -> X -> M in a cubic cell of a = 1 bohr: two segments of length
    # pi; 12 requested points give a spacing of 2 pi / 11, so int(5.5) = 5
    # steps per segment: 4 interior points and the end point, 11 points.
    paths = [np.array([[0, 0, 0], [0.5, 0, 0], [0.5, 0.5, 0]])]
    k, mag, w, idx = band.path_kpoints(_cubic(), paths, 12)
    assert len(k) == 11 and idx == [1, 6, 11]
    frac = band.to_fractional(_cubic(), k)
    expect = np.array([[0.1 * i, 0, 0] for i in range(6)] + [[0.5, 0.1 * i, 0] for i in range(1, 6)])
    assert np.allclose(frac, expect)
    assert np.allclose(mag, np.arange(11) * math.pi / 5)
    assert np.allclose(w, 2.0 / 11)


def test_second_path_restarts_at_the_same_distance():
    paths = [np.array([[0, 0, 0], [0.5, 0, 0]]), np.array([[0, 0, 0.5], [0, 0, 0]])]
    k, mag, _, idx = band.path_kpoints(_cubic(), paths, 4)
    # num_path_kp equals the number of high-symmetry points: the points alone
    assert np.allclose(mag, [0.0, math.pi, math.pi, 2.0 * math.pi])
    k, mag, _, idx = band.path_kpoints(_cubic(), paths, 9)
    # spacing 2 pi / 8: int(4) = 4 steps on the first path; the second path's
    # first point repeats the distance where the first path ended, and its 4
    # steps would pass the 9 requested points, so they are cut to 3
    assert idx == [1, 5, 6, 9]
    assert np.allclose(mag / math.pi, [0, 0.25, 0.5, 0.75, 1, 1, 4 / 3, 5 / 3, 2])
    assert np.allclose(band.to_fractional(_cubic(), k[5:]),
                       [[0, 0, 0.5], [0, 0, 1 / 3], [0, 0, 1 / 6], [0, 0, 0]])


def test_segment_without_steps_keeps_the_previous_step():
    # a short final segment with int(d / spacing) = 0: no interior points, and
    # its end point's distance adds the previous segment's step, as the
    # reference's segmentDelta keeps its value
    paths = [np.array([[0, 0, 0], [0.5, 0, 0], [0.5, 0.01, 0]])]
    k, mag, _, idx = band.path_kpoints(_cubic(), paths, 6)
    step = (math.pi + 0.02 * math.pi) / 5
    n1 = int(math.pi / step)
    assert idx == [1, n1 + 1, n1 + 2]
    assert mag[-1] == pytest.approx(mag[-2] + math.pi / n1)
