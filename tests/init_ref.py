"""Restatement of the device initialisers (checker): Philox4x64-10
(Salmon et al., SC 2011) in Python integers, and the catalogue setters of
app/PositionSetterProvider.java, app/TypeSetterProvider.java and
app/MatrixGeneratorProvider.java on its draws."""
import math

import numpy as np

M0, M1 = 0xD2E7470EE14C6C93, 0xCA5A826395121157
W0, W1 = 0x9E3779B97F4A7C15, 0xBB67AE8584CAA73B
MASK = (1 << 64) - 1


def philox4x64(c, k):
    c = list(c)
    k = list(k)
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 64) ^ c[1] ^ k[0], p1 & MASK, (p0 >> 64) ^ c[3] ^ k[1], p0 & MASK]
        k = [(k[0] + W0) & MASK, (k[1] + W1) & MASK]
    return c


def unit(w):
    return (w >> 11) * 2.0 ** -53


def normal(u1, u2):
    return math.sqrt(-2.0 * math.log(1.0 - u1)) * math.cos(2.0 * math.pi * u2)


def ensure(x, wrap):
    if wrap:
        x = x - math.floor(x)
        return 0.0 if x >= 1.0 else x
    return min(max(x, 0.0), 1.0)


def map_type(v, n):
    return max(0, min(n - 1, int(math.floor(v * n))))


F03, F05, F01, F02, F015 = (float(np.float32(x)) for x in (0.3, 0.5, 0.1, 0.2, 0.15))


def position(setter, seed, i, t, n):
    u0, u1, u2, u3 = (unit(w) for w in philox4x64([i, 0, 0, 0], [seed, 0]))
    tp = 2.0 * math.pi
    if setter == 0:
        return u0, u1
    if setter == 1:
        x, y = normal(u0, u1) * F03, normal(u2, u3) * F03
    elif setter == 2:
        a, r = u0 * tp, 0.5 * math.sqrt(u1)
        x, y = math.cos(a) * r, math.sin(a) * r
    elif setter == 3:
        a, r = u0 * tp, F05 * u1
        x, y = math.cos(a) * r, math.sin(a) * r
    elif setter == 4:
        a, r = u0 * tp, 0.7 + 0.02 * normal(u2, u3)
        x, y = math.cos(a) * r, math.sin(a) * r
    elif setter == 5:
        a, r = (0.3 * normal(u0, u1) + t) / n * tp, 0.7 + 0.02 * normal(u2, u3)
        x, y = math.cos(a) * r, math.sin(a) * r
    elif setter == 6:
        ca, a, r = t / n * tp, u0 * tp, u1 * F01
        x, y = F05 * math.cos(ca) + math.cos(a) * r, F05 * math.sin(ca) + math.sin(a) * r
    elif setter == 7:
        ca = t / n * tp
        x, y = F03 * math.cos(ca) + normal(u0, u1) * F02, F03 * math.sin(ca) + normal(u2, u3) * F02
    elif setter == 8:
        x, y = 2 * u0 - 1, (2 * u1 - 1) * F015
    elif setter == 9:
        f = u0
        a, sp = 2.0 * tp * f, 0.5 * min(f, 0.2)
        r = 0.9 * f + sp * normal(u2, u3) * sp
        x, y = r * math.cos(a), r * math.sin(a)
    else:
        f = (t + 1) / (n + 2) + 0.3 / n * normal(u0, u1)
        f = min(max(f, 0.0), 1.0)
        a, sp = 2.0 * tp * f, 0.5 * min(f, 0.2)
        r = 0.9 * f + sp * normal(u2, u3) * sp
        x, y = r * math.cos(a), r * math.sin(a)
    return x * 0.5 + 0.5, y * 0.5 + 0.5


def type_of(setter, seed, i, pos, vel, t, n):
    v0, v1 = (unit(w) for w in philox4x64([i, 1, 0, 0], [seed, 0])[:2])
    if setter == 0:
        return int(math.floor(v0 * n))
    if setter == 1:
        return map_type(v1, n) if v0 < 0.1 else t
    if setter == 2:
        return map_type(pos[0], n)
    if setter == 3:
        dx, dy, dz = pos[0] - 0.5, pos[1] - 0.5, pos[2]
        return map_type(math.sqrt(dx * dx + (dy * dy + dz * dz)) * 2, n)
    if setter == 4:
        return (t + 1) % n
    if setter == 5:
        return n - 1 - t
    if setter == 6:
        return map_type(v0 * v1, n)
    return n - 1 if math.sqrt(vel[0] ** 2 + (vel[1] ** 2 + vel[2] ** 2)) < 0.01 else t


def matrix(kind, size, seed):
    m = np.zeros((size, size))
    for i in range(size):
        for j in range(size):
            diag, nxt, prv = j == i, j == (i + 1) % size, j == (i + size - 1) % size
            if kind in (0, 1):
                m[i, j] = 2 * unit(philox4x64([i * size + j, 3, 0, 0], [seed, 0])[0]) - 1
            elif kind == 2:
                m[i, j] = 1.0 if (diag or nxt or prv) else -1.0
            elif kind == 3:
                m[i, j] = 1.0 if diag else (0.2 if (nxt or prv) else -1.0)
            elif kind == 4:
                m[i, j] = 1.0 if diag else (0.2 if (nxt or prv) else 0.0)
            elif kind == 5:
                m[i, j] = 1.0 if diag else (0.2 if nxt else 0.0)
    if kind == 1:
        for i in range(size):
            for j in range(i, size):
                m[i, j] = m[j, i]
    return m
