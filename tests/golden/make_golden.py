"""Generates the golden vectors in this directory.

A second, independent restatement of the reference's physics step, written
as literal pure-Python loops over Python floats (IEEE double, no fused
multiply-add), following tom-mohr/particle-life-app
(src/main/java/com/particle_life/):

  backend/Physics.java:309-354  makeContainers      -> make_containers()
  backend/Physics.java:362-375  getContainerIndex   -> container_index()
  backend/Physics.java:377-395  wrapContainerX/Y    -> wrap_container()
  backend/Physics.java:397-441  updateVelocity      -> update_velocity()
  backend/Physics.java:443-450  updatePosition      -> update_position()
  backend/Range.java:40-96      wrap/wrapConnection/clamp
  app/Main.java:275-280         the default Accelerator

The C oracle (oracle/plg_oracle.c) is checked against these vectors by
tests/test_golden.py.  The reference itself cannot run here (Java 21 + JOML,
no JDK), so the vectors pin the oracle to this restatement, not to the
reference's own output.  Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def range_wrap(v: float) -> float:
    if v < 0:
        while True:
            v += 1
            if not v < 0:
                break
        return v
    while v >= 1:
        v -= 1
    return v


def wrap_connection(v: float) -> float:
    if v < -0.5:
        return v + 1
    if v >= 0.5:
        return v - 1
    return v


def range_clamp(v: float) -> float:
    return 0.0 if v < 0 else (1.0 if v > 1 else v)


def accelerate(a: float, beta: float, pos: list) -> list:
    dist = math.sqrt(pos[0] * pos[0] + (pos[1] * pos[1] + pos[2] * pos[2]))
    force = (dist / beta - 1) if dist < beta else a * (1 - abs(1 + beta - 2 * dist) / (1 - beta))
    k = force / dist
    return [pos[0] * k, pos[1] * k, pos[2] * k]


def mix64(i: int) -> int:
    m = (1 << 64) - 1
    z = (i + 0x9E3779B97F4A7C15) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    return z ^ (z >> 31)


class World:
    def __init__(self, dim, pos, vel, types, matrix, rmax, friction, force, dt, beta, wrap):
        self.dim = dim
        self.pos = [list(map(float, p)) for p in pos]
        self.vel = [list(map(float, v)) for v in vel]
        self.types = [int(t) for t in types]
        self.ids = list(range(len(self.pos)))
        self.m = [list(map(float, r)) for r in matrix]
        self.rmax, self.friction, self.force, self.dt, self.beta, self.wrap = rmax, friction, force, dt, beta, wrap

    def container_index(self, p, cs, nx):
        c = []
        for k in range(self.dim):
            ck = int(p[k] / cs)
            if ck == nx:
                ck = nx - 1
            c.append(ck)
        idx = c[0] + c[1] * nx
        if self.dim == 3:
            idx += c[2] * nx * nx
        return idx

    def make_containers(self, cs, nx):
        n = len(self.pos)
        ncell = nx ** self.dim
        containers = [0] * ncell
        cell = [self.container_index(p, cs, nx) for p in self.pos]
        for c in cell:
            containers[c] += 1
        offset = 0
        for c in range(ncell):
            cap = containers[c]
            containers[c] = offset
            offset += cap
        order = [0] * n
        for i in range(n):
            order[containers[cell[i]]] = i
            containers[cell[i]] += 1
        self.pos = [self.pos[i] for i in order]
        self.vel = [self.vel[i] for i in order]
        self.types = [self.types[i] for i in order]
        self.ids = [self.ids[i] for i in order]
        return containers, [cell[i] for i in order]

    @staticmethod
    def wrap_container(c, n):
        if c < 0:
            return c + n
        if c >= n:
            return c - n
        return c

    def step(self):
        cs = self.rmax
        nx = int(math.floor(1 / cs))
        containers, cells = self.make_containers(cs, nx)
        n = len(self.pos)
        pairs = [0] * n
        hsum = [0] * n
        hxor = [0] * n
        acc = [[0.0, 0.0, 0.0] for _ in range(n)]
        zr = (-1, 0, 1) if self.dim == 3 else (0,)
        for i in range(n):
            p = self.pos[i]
            v = self.vel[i]
            ff = math.pow(self.friction, 60 * self.dt)
            v[0] = v[0] * ff
            v[1] = v[1] * ff
            v[2] = v[2] * ff
            c0 = [int(math.floor(p[k] / cs)) for k in range(self.dim)]
            for oz in zr:
                for oy in (-1, 0, 1):
                    for ox in (-1, 0, 1):
                        cx = self.wrap_container(c0[0] + ox, nx)
                        cy = self.wrap_container(c0[1] + oy, nx)
                        cz = self.wrap_container(c0[2] + oz, nx) if self.dim == 3 else 0
                        if self.wrap:
                            cx = self.wrap_container(cx, nx)
                            cy = self.wrap_container(cy, nx)
                            if self.dim == 3:
                                cz = self.wrap_container(cz, nx)
                        elif not (0 <= cx < nx and 0 <= cy < nx and 0 <= cz < nx):
                            continue
                        ci = cx + cy * nx + cz * nx * nx
                        start = 0 if ci == 0 else containers[ci - 1]
                        stop = containers[ci]
                        for j in range(start, stop):
                            if i == j:
                                continue
                            q = self.pos[j]
                            r = [q[0] - p[0], q[1] - p[1], (q[2] - p[2]) if self.dim == 3 else 0.0]
                            if self.wrap:
                                r = [wrap_connection(r[0]), wrap_connection(r[1]),
                                     wrap_connection(r[2]) if self.dim == 3 else 0.0]
                            d2 = r[0] * r[0] + (r[1] * r[1] + r[2] * r[2])
                            if d2 != 0 and d2 <= self.rmax * self.rmax:
                                r = [r[0] / self.rmax, r[1] / self.rmax, r[2] / self.rmax]
                                dv = accelerate(self.m[self.types[i]][self.types[j]], self.beta, r)
                                scale = self.rmax * self.force * self.dt
                                for k in range(3):
                                    acc[i][k] += dv[k]
                                    v[k] = v[k] + dv[k] * scale
                                pairs[i] += 1
                                h = mix64(self.ids[j])
                                hsum[i] = (hsum[i] + h) & ((1 << 64) - 1)
                                hxor[i] ^= h
        for i in range(n):
            p, v = self.pos[i], self.vel[i]
            for k in range(3):
                p[k] = v[k] * self.dt + p[k]
            if self.wrap:
                p[0], p[1] = range_wrap(p[0]), range_wrap(p[1])
                p[2] = range_wrap(p[2]) if self.dim == 3 else 0.0
            else:
                p[0], p[1] = range_clamp(p[0]), range_clamp(p[1])
                p[2] = range_clamp(p[2]) if self.dim == 3 else 0.0
        return dict(cell=cells, pairs=pairs, hsum=hsum, hxor=hxor, acc=[a[: self.dim] for a in acc])


CASES = {
    # name: (dim, n, ntypes, rmax, wrap, dt, seed, vel_scale)
    "wrap2d": (2, 400, 5, 0.1, True, 0.02, 1, 0.05),
    "clamp2d": (2, 300, 4, 0.08, False, 0.02, 2, 0.2),
    "sliver2d": (2, 300, 3, 0.13, True, 0.02, 3, 0.05),
    "nx2_2d": (2, 60, 3, 0.4, True, 0.02, 4, 0.05),
    "nx1_2d_clamp": (2, 40, 2, 0.7, False, 0.02, 5, 0.05),
    "wrap3d": (3, 300, 4, 0.2, True, 0.01, 6, 0.05),
}
STEPS = 3
FRICTION = 0.5 ** (1.0 / (60.0 * 0.043))


def inputs(dim, n, ntypes, seed, vel_scale):
    rng = np.random.Generator(np.random.Philox(seed))
    pos = np.zeros((n, 3))
    pos[:, :dim] = rng.random((n, dim), dtype=np.float32)
    vel = np.zeros((n, 3))
    vel[:, :dim] = np.asarray(rng.standard_normal((n, dim)) * vel_scale, np.float32)
    types = rng.integers(0, ntypes, n).astype(np.int32)
    m = np.asarray(2 * rng.random((ntypes, ntypes)) - 1, np.float32).astype(np.float64)
    return pos, vel, types, m


def main():
    for name, (dim, n, nt, rmax, wrap, dt, seed, vs) in CASES.items():
        pos, vel, types, m = inputs(dim, n, nt, seed, vs)
        w = World(dim, pos, vel, types, m, rmax, FRICTION, 1.0, dt, 0.3, wrap)
        out = dict(in_pos=pos, in_vel=vel, in_types=types, matrix=m,
                   params=np.array([dim, rmax, FRICTION, 1.0, dt, 0.3, 1.0 if wrap else 0.0]))
        for s in range(STEPS):
            d = w.step()
            out[f"cell{s}"] = np.array(d["cell"], np.int32)
            out[f"pairs{s}"] = np.array(d["pairs"], np.int32)
            out[f"hsum{s}"] = np.array(d["hsum"], np.uint64)
            out[f"hxor{s}"] = np.array(d["hxor"], np.uint64)
            out[f"acc{s}"] = np.array(d["acc"], np.float64)
            out[f"pos{s}"] = np.array(w.pos, np.float64)
            out[f"vel{s}"] = np.array(w.vel, np.float64)
            out[f"ids{s}"] = np.array(w.ids, np.int32)
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, "pairs/particle", float(np.mean(out["pairs0"])))


if __name__ == "__main__":
    main()
