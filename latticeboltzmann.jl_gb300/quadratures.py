"""Velocity sets (quadratures) of LatticeBoltzmann.jl: D2Q4, D2Q5, D2Q9, D2Q13, D2Q17,
D2Q21 (25 velocities) and D2Q37.

Each class holds the reference's three fields (src/quadratures/D2Q*.jl):
``abscissae`` (2 x Q integer matrix), ``weights`` and ``speed_of_sound_squared`` -- which,
as in the reference, holds 1 / c_s^2 (e.g. 3.0 for D2Q9, D2Q9.jl:26).  ``order(q)`` and
``opposite(q, idx)`` follow src/quadratures.jl:11-19 and the per-set overrides; ``opposite``
keeps the reference's 1-based indices, ``q.opposites`` is the 0-based array.
"""
from __future__ import annotations

import math

import numpy as np


class Quadrature:
    name = "Quadrature"
    _order = 0
    qid = -1

    def __init__(self, abscissae, weights, speed_of_sound_squared):
        self.abscissae = np.asarray(abscissae, dtype=np.int64)
        self.weights = np.asarray(weights, dtype=np.float64)
        self.speed_of_sound_squared = float(speed_of_sound_squared)
        self.opposites = np.array([opposite(self, i + 1) - 1 for i in range(len(self.weights))], dtype=np.int64)

    @property
    def Q(self) -> int:
        return len(self.weights)

    def __repr__(self):
        return self.name

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(self.name)


def dimension(q: Quadrature) -> int:
    return 2


def order(q: Quadrature) -> int:
    return q._order


def opposite(q: Quadrature, idx: int) -> int:
    """1-based index of the abscissa opposite to `idx` (src/quadratures.jl:11-19 and the
    D2Q4 / D2Q5 / D2Q9 overrides, D2Q4.jl:26-31, D2Q5.jl:34-42, D2Q9.jl:30-38)."""
    if isinstance(q, D2Q4):
        return idx + 2 if idx <= 2 else idx - 2
    if isinstance(q, D2Q5):
        if idx == 1:
            return 1
        return idx + 2 if idx <= 3 else idx - 2
    if isinstance(q, D2Q9):
        if idx == 1:
            return 1
        return idx + 4 if idx <= 5 else idx - 4
    if idx == 1:
        return 1
    return idx + 1 if idx % 2 == 0 else idx - 1


class D2Q4(Quadrature):
    name, _order, qid = "D2Q4", 3, 0

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        super().__init__([[1, 0, -1, 0], [0, 1, 0, -1]], [1 / 4, 1 / 4, 1 / 4, 1 / 4], 2.0)


class D2Q5(Quadrature):
    name, _order, qid = "D2Q5", 3, 1

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        super().__init__([[0, 1, 0, -1, 0], [0, 0, 1, 0, -1]], [4 / 6, 1 / 12, 1 / 12, 1 / 12, 1 / 12], 6.0)


class D2Q9(Quadrature):
    name, _order, qid = "D2Q9", 5, 2

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        super().__init__([[0, -1, -1, -1, 0, 1, 1, 1, 0], [0, 1, 0, -1, -1, -1, 0, 1, 1]],
                         [4 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9, 1 / 36, 1 / 9], 3.0)


class D2Q13(Quadrature):
    name, _order, qid = "D2Q13", 5, 3

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        w0, w1, w2, w3 = 3 / 8, 1 / 12, 1 / 16, 1 / 96
        super().__init__([[0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0],
                          [0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, -2, 2]],
                         [w0, w1, w1, w1, w1, w2, w2, w2, w2, w3, w3, w3, w3], 2.0)


class D2Q17(Quadrature):
    name, _order, qid = "D2Q17", 7, 4

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        sq = math.sqrt(193)
        w0 = (575 + 193 * sq) / 8100
        w1 = (3355 - 91 * sq) / 18000
        w2 = (655 + 17 * sq) / 27000
        w3 = (685 - 49 * sq) / 54000
        w4 = (1445 - 101 * sq) / 162000
        super().__init__([[0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 2, -2, 3, -3, 0, 0],
                          [0, 0, 0, 1, -1, 1, -1, -1, 1, 2, -2, -2, 2, 0, 0, 3, -3]],
                         [w0] + [w1] * 4 + [w2] * 4 + [w3] * 4 + [w4] * 4,
                         (125 + 5 * math.sqrt(193)) / 72)


class D2Q21(Quadrature):
    name, _order, qid = "D2Q21", 7, 5

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        w = [91 / 324] + [1 / 12] * 4 + [2 / 27] * 4 + [7 / 360] * 4 + [1 / 432] * 4 + [1 / 1620] * 4 + [0.0] * 4
        super().__init__(
            [[0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, 2, -2, 3, -3, 0, 0, 3, -3, -3, 3],
             [0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 2, -2, -2, 2, 0, 0, 3, -3, 3, -3, 3, -3]],
            w, 3 / 2)


class D2Q37(Quadrature):
    name, _order, qid = "D2Q37", 9, 6

    def __init__(self, *args):
        if args:
            return super().__init__(*args)
        g = [0.23315066913235250228650, 0.10730609154221900241246, 0.05766785988879488203006,
             0.01420821615845075026469, 0.00535304900051377523273, 0.00101193759267357547541,
             0.00024530102775771734547, 0.00028341425299419821740]
        w = [g[0]] + [g[1]] * 4 + [g[2]] * 4 + [g[3]] * 4 + [g[4]] * 8 + [g[5]] * 4 + [g[6]] * 4 + [g[7]] * 8
        r = 1.19697977039307435897239
        super().__init__(
            [[0, 1, -1, 0, 0, 1, -1, 1, -1, 2, -2, 0, 0, 2, -2, -2, 2, 1, -1, 1, -1, 2, -2, 2, -2,
              3, -3, 0, 0, 3, -3, 3, -3, 1, -1, -1, 1],
             [0, 0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 2, -2, 1, -1, 1, -1, 2, -2, -2, 2, 2, -2, -2, 2,
              0, 0, 3, -3, 1, -1, -1, 1, 3, -3, 3, -3]],
            w, r * r)


# the reference's `Quadratures` named tuple (src/quadratures.jl:30-38)
Quadratures = {"D2Q4": D2Q4(), "D2Q5": D2Q5(), "D2Q9": D2Q9(), "D2Q13": D2Q13(), "D2Q17": D2Q17(),
               "D2Q21": D2Q21(), "D2Q37": D2Q37()}
