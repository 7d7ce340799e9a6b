"""Save / load of a world in the app's save layout (app/Main.java:1258-1348).

A save is a zip archive with
  particles.tsv  header ``x\\ty\\tvx\\tvy\\tcolor``, one particle per line
                 (app/io/ParticlesIO.java:8-46); 2D only in the app.  3D
                 worlds of this library write ``x\\ty\\tz\\tvx\\tvy\\tvz\\tcolor``
                 (an extension; the 2D layout is unchanged)
  physics.toml   ``boundaries`` ("periodic" | "clamped"), ``radius``,
                 ``friction``, ``force`` (app/PhysicsSettingsToml.java:9-33;
                 dt is not saved)
  matrix.tsv     one row of the matrix per line, tab-separated
                 (app/io/MatrixIO.java:10-42)
  img.png        optional thumbnail (ignored on load, as in the app)
Doubles are written the way Java's ``Double.toString`` writes them (the
shortest decimal that reads back to the same double, plain notation for
1e-3 <= |x| < 1e7, otherwise ``d.dddE<exp>``), so saves are byte-compatible
with the app's and every value round-trips exactly.  Missing entries load
as None: the app then keeps its current state for that part.
"""
from __future__ import annotations

import io
import math
import struct
import tomllib
import zipfile
import zlib
from dataclasses import dataclass
from typing import Optional

import numpy as np

PARTICLES = "particles.tsv"
SETTINGS = "physics.toml"
MATRIX = "matrix.tsv"
IMAGE = "img.png"


def java_double(x: float) -> str:
    """Java's Double.toString of a double (JDK 19+ shortest-digits rule)."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign = "-" if x < 0 else ""
    # shortest round-trip digits and decimal exponent from repr
    mant, _, exp = repr(abs(x)).partition("e")
    e10 = int(exp) if exp else 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    point = len(ip) + e10  # position of the decimal point relative to the digit string start
    lead_zeros = len(ip + fp) - len((ip + fp).lstrip("0"))
    point -= lead_zeros
    digits = digits.rstrip("0") or "0"
    a = abs(x)
    if 1e-3 <= a < 1e7:
        if point <= 0:
            return sign + "0." + "0" * (-point) + digits
        if point >= len(digits):
            return sign + digits + "0" * (point - len(digits)) + ".0"
        return sign + digits[:point] + "." + digits[point:]
    frac = digits[1:] or "0"
    return f"{sign}{digits[0]}.{frac}E{point - 1}"


@dataclass
class SavedState:
    positions: Optional[np.ndarray]   # (n, 3) float64, z = 0 in 2D
    velocities: Optional[np.ndarray]  # (n, 3) float64
    types: Optional[np.ndarray]       # (n,) int32
    wrap: Optional[bool]
    rmax: Optional[float]
    friction: Optional[float]
    force: Optional[float]
    matrix: Optional[np.ndarray]      # (t, t) float64
    dim: int = 2


def particles_tsv(positions: np.ndarray, velocities: np.ndarray, types: np.ndarray, dim: int = 2) -> str:
    """ParticlesIO.saveParticles (app/io/ParticlesIO.java:31-46)."""
    p = np.asarray(positions, np.float64).reshape(-1, 3)
    v = np.asarray(velocities, np.float64).reshape(-1, 3)
    t = np.asarray(types, np.int64)
    out = ["x\ty\tvx\tvy\tcolor" if dim == 2 else "x\ty\tz\tvx\tvy\tvz\tcolor"]
    for i in range(p.shape[0]):
        cols = [p[i, k] for k in range(dim)] + [v[i, k] for k in range(dim)]
        out.append("\t".join(java_double(c) for c in cols) + f"\t{int(t[i])}")
    return "\n".join(out) + "\n"


def parse_particles(text: str):
    """ParticlesIO.loadParticles (app/io/ParticlesIO.java:8-29): skips the
    header; 2D rows are x, y, vx, vy, type (z = 0)."""
    lines = text.splitlines()
    header = lines[0].split("\t") if lines else []
    dim = 3 if "z" in header else 2
    rows = [ln.split("\t") for ln in lines[1:] if ln.strip()]
    n = len(rows)
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    typ = np.zeros(n, np.int32)
    for i, r in enumerate(rows):
        for k in range(dim):
            pos[i, k] = float(r[k])
            vel[i, k] = float(r[dim + k])
        typ[i] = int(r[2 * dim])
    return pos, vel, typ, dim


def matrix_tsv(m: np.ndarray) -> str:
    """MatrixIO.saveMatrix (app/io/MatrixIO.java:27-42)."""
    m = np.asarray(m, np.float64)
    return "".join("\t".join(java_double(x) for x in row) + "\n" for row in m)


def parse_matrix(text: str) -> np.ndarray:
    """MatrixIO.loadMatrix (app/io/MatrixIO.java:10-25): square, size = rows."""
    rows = [[float(x) for x in ln.split("\t")] for ln in text.splitlines() if ln.strip()]
    t = len(rows)
    return np.array([r[:t] for r in rows], np.float64).reshape(t, t)


def settings_toml(wrap: bool, rmax: float, friction: float, force: float) -> str:
    """PhysicsSettingsToml.fromPhysicsSettings (app/PhysicsSettingsToml.java:18-25)."""
    return (f'boundaries = "{"periodic" if wrap else "clamped"}"\n'
            f"radius = {java_double(rmax)}\n"
            f"friction = {java_double(friction)}\n"
            f"force = {java_double(force)}\n")


def parse_settings(text: str) -> dict:
    """PhysicsSettingsToml.toPhysicsSettings (app/PhysicsSettingsToml.java:27-33),
    with the file's defaults for missing keys (lines 10-17)."""
    t = tomllib.loads(text)
    return {"wrap": t.get("boundaries", "periodic") == "periodic", "rmax": float(t.get("radius", 0.02)),
            "friction": float(t.get("friction", 0.85)), "force": float(t.get("force", 1.0))}


THUMBNAIL_SIZE = 256  # Main.SAVE_IMAGE_SIZE (app/Main.java:168)


def png_rgba(rows) -> bytes:
    """An 8-bit RGBA PNG of a (height, width, 4) uint8 array; row 0 of the
    array is the first row of the file.  The app stores glReadPixels rows
    (bottom of the framebuffer first) unchanged (app/Main.java:1279-1289),
    so plg_render's rows go in as they come."""
    a = np.ascontiguousarray(rows, np.uint8)
    h, w = a.shape[:2]

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    raw = b"".join(b"\x00" + a[j].tobytes() for j in range(h))  # filter type 0 per row
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def read_png_rgba(data: bytes) -> np.ndarray:
    """Reads back what png_rgba writes (8-bit RGBA, filter type 0 rows)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    off, idat, w, h = 8, b"", 0, 0
    while off < len(data):
        (ln,) = struct.unpack(">I", data[off:off + 4])
        kind, body = data[off + 4:off + 8], data[off + 8:off + 8 + ln]
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 8 or ctype != 6:
                raise ValueError("only 8-bit RGBA")
        elif kind == b"IDAT":
            idat += body
        off += 12 + ln
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    if np.any(raw[:, 0] != 0):
        raise ValueError("only filter type 0")
    return raw[:, 1:].reshape(h, w, 4).copy()


def save_state(path, positions, velocities, types, *, wrap: bool, rmax: float, friction: float, force: float,
               matrix, dim: int = 2, image_png: Optional[bytes] = None) -> None:
    """Main.saveState (app/Main.java:1258-1297)."""
    with zipfile.ZipFile(path, "w", compression=zipfile.ZIP_DEFLATED) as z:
        z.writestr(PARTICLES, particles_tsv(positions, velocities, types, dim))
        z.writestr(SETTINGS, settings_toml(wrap, rmax, friction, force))
        z.writestr(MATRIX, matrix_tsv(matrix))
        if image_png is not None:
            z.writestr(IMAGE, image_png)


def load_state(path) -> SavedState:
    """Main.loadState (app/Main.java:1314-1348): entries that are missing
    come back as None; unknown entries are ignored."""
    st = SavedState(None, None, None, None, None, None, None, None)
    with zipfile.ZipFile(path, "r") as z:
        names = set(z.namelist())
        if PARTICLES in names:
            st.positions, st.velocities, st.types, st.dim = parse_particles(z.read(PARTICLES).decode())
        if SETTINGS in names:
            s = parse_settings(z.read(SETTINGS).decode())
            st.wrap, st.rmax, st.friction, st.force = s["wrap"], s["rmax"], s["friction"], s["force"]
        if MATRIX in names:
            st.matrix = parse_matrix(z.read(MATRIX).decode())
    return st


def save_bytes(**kw) -> bytes:
    buf = io.BytesIO()
    save_state(buf, **kw)
    return buf.getvalue()
