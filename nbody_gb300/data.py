"""Body data: the host-side counterpart of the reference's `nbody_data`.

Mirrors nbody/nbody_data.h (bodies, time, step, the G1 table load/save of
the reference's golden vectors, make_universe) and adds the seeded synthetic
inputs the GB300 engine is measured on (uniform cube, Plummer sphere).  Everything here is input preparation on the
host; forces and conservation sums run on the GPU through the engine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MIN_DISTANCE = 1e-8  # nbody/nbtype.h:79, compared with r^2
BLOCK_SIZE = 64      # nbody/nbtype.h:77 NBODY_DATA_BLOCK_SIZE



@dataclass
class NBodyData:
    """Bodies in AoS form, like nbody/nbody_data.h:9-35."""

    vertices: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    velocities: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    mass: np.ndarray = field(default_factory=lambda: np.zeros(0))
    radius: np.ndarray = field(default_factory=lambda: np.zeros(0))
    color: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), dtype=np.float32))
    time: float = 0.0
    step: int = 0
    box_size: int = 0
    check_list: str = "PLVE"
    _initial: dict = field(default=None, repr=False)
    _last: dict = field(default=None, repr=False)
    _prev_compute_count: int = field(default=0, repr=False)

    # -- nbody/nbody_data.cpp:176-212 ----------------------------------------
    def get_color(self) -> np.ndarray:
        """Colours (N x 4 float32); white where none were given, as the
        reference's loaders set them (nbody/nbody_data.cpp:508,613)."""
        n = self.get_count()
        if self.color.shape != (n, 4):
            self.color = np.ones((n, 4), dtype=np.float32)
        return self.color

    def get_count(self) -> int:
        return int(self.mass.size)

    def advise_time(self, dt: float) -> None:
        self.time += dt
        self.step += 1

    def get_time(self) -> float:
        return self.time

    def set_time(self, t: float) -> None:
        self.time = float(t)

    def get_step(self) -> int:
        return self.step

    def set_step(self, s: int) -> None:
        self.step = int(s)

    # -- conservation check: nbody/nbody_data.cpp:57-145, 366-381 -------------
    def set_check_list(self, check_list: str) -> None:
        """Which of P, L, V, E print_statistics computes."""
        self.check_list = check_list

    def print_statistics(self, engine=None) -> str:
        """The reference's conservation line: step, time, compute counts and
        the drifts of momentum (dP, %), angular momentum (dL, %), mass-centre
        speed (Vcm) and energy (dE, %) against the first call.  The sums are
        the engine's FP64 GPU reductions of its current state (nbg_statistics)
        instead of the reference's host sums after get_data; the bodies are
        still fetched into this object, as the reference does.  Returns the
        line (also printed)."""
        cc = 0
        if engine is not None:
            engine.get_data(self)
            cc = engine.get_compute_count()
            st = engine.statistics()
        else:
            raise ValueError("print_statistics needs the engine that holds the state")
        now = {"P": st[0:3].copy(), "L": st[3:6].copy(), "KE": float(st[6]),
               "PE": float(st[7]), "V": st[8:11].copy()}
        if self._initial is None:
            self._initial = now
        self._last = now
        parts = [f"#{self.step:08d}", f"t {self.time:.6f}", f"CC {cc:08d}",
                 f"SC {cc - self._prev_compute_count:8d}"]
        self._prev_compute_count = cc
        if "P" in self.check_list:
            parts.append(f"dP {self.get_impulce_err():.3e}")
        if "L" in self.check_list:
            parts.append(f"dL {self.get_impulce_moment_err():.3e}")
        if "V" in self.check_list:
            vcm = (self._last["V"] - self._initial["V"]) / self.time if self.time else \
                np.zeros(3)
            parts.append(f"Vcm {np.linalg.norm(vcm):.3e}")
        if "E" in self.check_list:
            parts.append(f"dE {self.get_energy_err():.3e}")
        line = " ".join(parts)
        print(line)
        return line

    def get_impulce_err(self) -> float:
        p0, p1 = self._initial["P"], self._last["P"]
        return abs(100.0 * np.linalg.norm(p1 - p0) / np.linalg.norm(p0))

    def get_impulce_moment_err(self) -> float:
        l0, l1 = self._initial["L"], self._last["L"]
        return abs(100.0 * np.linalg.norm(l1 - l0) / np.linalg.norm(l0))

    def get_energy_err(self) -> float:
        e0 = self._initial["KE"] + self._initial["PE"]
        e1 = self._last["KE"] + self._last["PE"]
        return abs(100.0 * (e1 - e0) / e0)

    # -- state vector helpers --------------------------------------------------
    def to_state(self) -> np.ndarray:
        """y = [rx | ry | rz | vx | vy | vz] (nbody/nbody_engine_simple.cpp:34-53)."""
        return np.concatenate([self.vertices.T.reshape(-1),
                               self.velocities.T.reshape(-1)]).astype(np.float64)

    def from_state(self, y: np.ndarray) -> None:
        n = self.get_count()
        y = np.asarray(y, dtype=np.float64)
        self.vertices = y[:3 * n].reshape(3, n).T.copy()
        self.velocities = y[3 * n:6 * n].reshape(3, n).T.copy()

    def is_equal(self, other: "NBodyData", eps: float = 0.0) -> bool:
        """nbody/nbody_data.cpp:389-411."""
        if self.get_count() != other.get_count():
            return False
        return bool(np.all(np.abs(self.mass - other.mass) <= eps)
                    and np.all(np.abs(self.radius - other.radius) <= eps)
                    and np.all(np.abs(self.vertices - other.vertices) <= eps)
                    and np.all(np.abs(self.velocities - other.velocities) <= eps))

    # -- text I/O: nbody/nbody_data.cpp:417-651 -------------------------------
    @classmethod
    def load(cls, path: str) -> "NBodyData":
        """The G1 table 'X Y Z Vx Vy Vz Mass [Radius] ...' with '//' comments
        (nbody/nbody_data.cpp:442-512), the format of the reference's golden
        vectors.  A malformed line raises ValueError where the reference
        returns false."""
        rows = []
        with open(path) as fh:
            for line_n, line in enumerate(fh):
                k = line.find("//")
                if k >= 0:
                    line = line[:k]
                cols = line.split()
                if not cols:
                    continue
                if len(cols) < 7:
                    raise ValueError(f"{path}:{line_n}: need at least 7 columns")
                vals = [float(c) for c in cols[:7]]
                vals.append(float(cols[7]) if len(cols) > 7 else 0.0)
                rows.append(vals)
        a = np.array(rows, dtype=np.float64).reshape(-1, 8)
        d = cls(vertices=a[:, 0:3].copy(), velocities=a[:, 3:6].copy(),
                mass=a[:, 6].copy(), radius=a[:, 7].copy())
        # nbody/nbody_data.cpp:640-651 (load_initial box size)
        r = np.maximum(np.max(a[:, 0:3], axis=0) if len(a) else 1.0, 1.0)
        d.box_size = int(np.max(r))
        return d

    def save(self, path: str) -> None:
        with open(path, "w") as fh:
            for i in range(self.get_count()):
                vals = list(self.vertices[i]) + list(self.velocities[i]) + [
                    self.mass[i], self.radius[i]]
                fh.write(" ".join(f"{v:+.16e}" for v in vals) + "\n")

    # -- generators -------------------------------------------------------------
    @classmethod
    def make_universe(cls, star_count: int, sx: float = 100.0, sy: float = 100.0,
                      sz: float = 100.0) -> "NBodyData":
        """Two rotating galaxies (nbody/nbody_data.cpp:263-324).

        Each galaxy holds round_up(star_count, 64) bodies: a central black hole
        of 0.999 of its mass and stars drawn from a mt19937_64 stream, as the
        reference does.  Used for the reference's engine tests (N = 128, 1024).
        """
        d = cls()
        radius = sx * 0.5
        galaxy_mass = 1000.0
        center = np.array([sx * 0.5, sy * 0.5, sz * 0.5])
        base = np.array([radius, 0.0, 0.0])
        f = _force(np.zeros(3), base, galaxy_mass, galaxy_mass)
        vel = np.array([0.0, math.sqrt(_length(f) * _length(base) / (2 * galaxy_mass)), 0.0])
        parts = [_galaxy(center - base, vel / 3, radius, galaxy_mass, star_count),
                 _galaxy(center + base, -vel / 3, radius, galaxy_mass, star_count)]
        d.vertices = np.concatenate([p[0] for p in parts])
        d.velocities = np.concatenate([p[1] for p in parts])
        d.mass = np.concatenate([p[2] for p in parts])
        d.radius = np.zeros(d.mass.size)
        # colours of nbody/nbody_data.cpp:278,315-320: the black hole green,
        # the stars of the two galaxies bluish and reddish
        k = np.float32(0.8)
        cols = []
        for p, c in zip(parts, ((k * 0.5, k * 0.5, k, 1.0), (k, k * 0.5, k * 0.5, 1.0))):
            col = np.tile(np.array(c, dtype=np.float32), (len(p[2]), 1))
            col[0] = (0.0, 1.0, 0.0, 1.0)
            cols.append(col)
        d.color = np.concatenate(cols).astype(np.float32)
        d.box_size = int(max(max(1.0, sx), max(sy, sz)))
        return d

    @classmethod
    def uniform_cube(cls, n: int, side: float = 100.0, seed: int = 1,
                     vel_sigma: float = 0.1) -> "NBodyData":
        """Positions U[-side/2, side/2]^3, v ~ N(0, vel_sigma), m ~ U[0.5,1.5]/n."""
        rng = np.random.default_rng(seed)
        d = cls(vertices=rng.uniform(-side / 2, side / 2, size=(n, 3)),
                velocities=rng.normal(0.0, vel_sigma, size=(n, 3)),
                mass=rng.uniform(0.5, 1.5, size=n) / n, radius=np.zeros(n))
        d.box_size = int(side)
        return d

    @classmethod
    def plummer(cls, n: int, seed: int = 1, scale: float = 1.0,
                total_mass: float = 1.0) -> "NBodyData":
        """Isotropic Plummer sphere, G = 1.

        Positions by inverting the cumulative mass M(r) = r^3 / (1 + r^2)^{3/2};
        speeds by von Neumann rejection of g(q) = q^2 (1 - q^2)^{7/2} times the
        local escape speed sqrt(2) (1 + r^2)^{-1/4} (the method of Aarseth,
        Henon & Wielen 1974).  Equal masses; centre of mass and momentum moved
        to the origin.  Radii are capped at 100 scale radii.
        """
        rng = np.random.default_rng(seed)
        x1 = rng.uniform(1e-10, 1.0, size=n)
        r = 1.0 / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
        bad = r > 100.0
        while np.any(bad):
            x1[bad] = rng.uniform(1e-10, 1.0, size=int(bad.sum()))
            r = 1.0 / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
            bad = r > 100.0
        pos = _iso(rng, n) * r[:, None]
        q = np.empty(n)
        todo = np.arange(n)
        while todo.size:
            qq = rng.uniform(0.0, 1.0, size=todo.size)
            gg = rng.uniform(0.0, 0.1, size=todo.size)
            ok = gg < qq * qq * (1.0 - qq * qq) ** 3.5
            q[todo[ok]] = qq[ok]
            todo = todo[~ok]
        vmag = q * math.sqrt(2.0) * (1.0 + r * r) ** (-0.25)
        vel = _iso(rng, n) * vmag[:, None]
        mass = np.full(n, total_mass / n)
        pos -= np.average(pos, axis=0, weights=mass)
        vel -= np.average(vel, axis=0, weights=mass)
        pos *= scale
        vel *= math.sqrt(total_mass / scale)
        d = cls(vertices=pos, velocities=vel, mass=mass, radius=np.zeros(n))
        d.box_size = int(max(1.0, np.max(np.abs(pos))))
        return d


def _iso(rng, n):
    """Uniform unit vectors."""
    z = rng.uniform(-1.0, 1.0, size=n)
    phi = rng.uniform(0.0, 2.0 * math.pi, size=n)
    s = np.sqrt(1.0 - z * z)
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def _norm2(v) -> float:
    """x x + y y + z z in the reference's order (nbody/vertex.h:151-158)."""
    x, y, z = float(v[0]), float(v[1]), float(v[2])
    return x * x + y * y + z * z


def _length(v) -> float:
    return math.sqrt(_norm2(v))


def _cross(a, b):
    """nbody/vertex.h:133-138."""
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]])


def _force(v1, v2, m1, m2):
    """nbody/nbody_data.cpp:35-44."""
    dr = v1 - v2
    r2 = _norm2(dr)
    r2 = max(r2, MIN_DISTANCE)
    return dr * ((-m1 * m2) / (r2 * math.sqrt(r2)))


class _MT19937_64:
    """64-bit Mersenne Twister (Matsumoto & Nishimura), default seed 5489,
    the engine behind std::mt19937_64 used by make_universe."""

    N, M = 312, 156
    MATRIX_A = 0xB5026F5AA96619E9
    UM, LM = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed: int = 5489):
        self.mt = [0] * self.N
        self.mt[0] = seed & self.MASK
        for i in range(1, self.N):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & self.MASK
        self.mti = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UM) | (mt[(i + 1) % self.N] & self.LM)
            xa = x >> 1
            if x & 1:
                xa ^= self.MATRIX_A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.mti = 0

    def __call__(self) -> int:
        if self.mti >= self.N:
            self._twist()
        x = self.mt[self.mti]
        self.mti += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        return x & self.MASK


def _galaxy(center, velocity, radius, total_mass, count):
    """nbody/nbody_data.cpp:218-261 (add_galaxy)."""
    rng = _MT19937_64()

    def uniform():
        # std::uniform_real_distribution<double>(-radius, radius) over a
        # 64-bit engine: one draw scaled by 2^-64.
        u = float(rng()) / 18446744073709551616.0
        return (radius - (-radius)) * u + (-radius)

    count = BLOCK_SIZE * (1 + (count - 1) // BLOCK_SIZE) - 1
    up = np.array([0.0, 0.0, 1.0])
    right = np.array([1.0, 0.0, 0.0])
    bh_mass = total_mass * 0.999
    star_mass = (total_mass - bh_mass) / count
    all_stars = count * star_mass
    pos = [np.array(center, dtype=np.float64)]
    vel = [np.array(velocity, dtype=np.float64)]
    mass = [bh_mass]
    n = 0
    while n != count:
        # nbvertex_t r(uniform(rng), uniform(rng), uniform(rng)): C++ leaves the
        # order of the three draws unspecified; g++ evaluates the constructor's
        # arguments last to first, so the first draw is z and the last is x
        # (checked against the reference's own build)
        u1, u2, u3 = uniform(), uniform(), uniform()
        r = np.array([u3, u2, u1])
        rlen = _length(r)
        if rlen > radius:
            continue
        r[2] *= 0.3
        r = r + center
        v = _cross(r - center, up)
        if _length(v) < 1e-7:
            v = _cross(r - center, right)
        v = v / _length(v)
        eff = (rlen / radius) ** 3.0 * all_stars + bh_mass
        fr = _force(r, center, star_mass, eff)
        v = v * math.sqrt(_length(fr) * _length(r - center) / star_mass)
        pos.append(r)
        vel.append(v + velocity)
        mass.append(star_mass)
        n += 1
    return np.array(pos), np.array(vel), np.array(mass)
