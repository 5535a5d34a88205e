"""Boundary conditions of LatticeBoltzmann.jl (src/boundary_conditions.jl and
src/boundary_conditions/*.jl), as descriptors for the fused device kernel.

  BounceBack(direction, xs, ys)          halfway bounce-back, bounce_back.jl:1-72
  MovingWall(North(), xs, ys, u[, ρ, T]) moving_wall.jl:1-38 (North only, as in the reference;
                                         like the reference it covers the whole top wall)

`xs` / `ys` are the reference's 1-based UnitRanges: give them as inclusive (lo, hi) tuples
or Python ranges over 1-based indices (range(1, NX + 1)).  The list order is the order in
which the rules overwrite populations (apply!, boundary_conditions.jl:6-20).
"""
from __future__ import annotations


class Direction:
    code = -1

    def __repr__(self):
        return type(self).__name__ + "()"

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self).__name__)


class North(Direction):
    code = 0


class East(Direction):
    code = 1


class South(Direction):
    code = 2


class West(Direction):
    code = 3


def _span(r):
    """(lo, hi) 1-based inclusive bounds of a tuple or a range of 1-based indices."""
    if isinstance(r, range):
        if len(r) == 0:
            return 1, 0
        if r.step != 1:
            raise ValueError("boundary ranges must be contiguous")
        return r.start, r.stop - 1
    lo, hi = r
    return int(lo), int(hi)


class BoundaryCondition:
    pass


class BounceBack(BoundaryCondition):
    def __init__(self, direction: Direction, xs, ys):
        self.direction = direction
        self.xs = _span(xs)
        self.ys = _span(ys)

    def __repr__(self):
        return f"BounceBack({self.direction!r}, {self.xs}, {self.ys})"


class MovingWall(BoundaryCondition):
    def __init__(self, direction: Direction, xs, ys, u, ρ=1.0, T=1.0):
        if not isinstance(direction, North):
            # the reference defines apply! for MovingWall{North} only (moving_wall.jl:17)
            raise NotImplementedError("MovingWall is provided for the North wall only")
        self.direction = direction
        self.xs = _span(xs)
        self.ys = _span(ys)
        self.u = [float(u[0]), float(u[1])]
        self.ρ = float(ρ)
        self.T = float(T)

    def __repr__(self):
        return f"MovingWall({self.direction!r}, {self.xs}, {self.ys}, {self.u})"
