"""pyref — a second, independent restatement of the reference GPU solver in pure Python
with numpy FP32 scalars, for tiny scenes only (it is slow).  Test infrastructure.

Written directly from the reference sources, with a different structure from the C
oracle (whole-array passes over Python lists of 3-tuples), so that a slip in one
restatement shows up as a difference between the two:
  Velvet/VtClothSolverGPU.hpp:56-111   Simulate schedule
  Velvet/VtClothSolverGPU.cu:42-465    kernels
  Velvet/VtClothSolverGPU.cuh:22-96    plane / sphere SDF, VelocityAt
  Velvet/SpatialHashGPU.cu:13-130      hash, cell ranges, neighbour cache
  Velvet/VtClothObjectGPU.hpp:75-147   grid constraints
Vector association follows glm (dot = (x*x + y*y) + z*z, mat4*vec4 = (c0*x + c1*y) +
(c2*z + c3*w)); acos is the same arcsin-series construction the oracle and the kernels
use (the reference's CUDA acosf cannot be reproduced bit for bit).
"""
from __future__ import annotations

import numpy as np

F = np.float32
EPS = F(1e-6)
ZERO = (F(0), F(0), F(0))


def add(a, b): return (a[0] + b[0], a[1] + b[1], a[2] + b[2])
def sub(a, b): return (a[0] - b[0], a[1] - b[1], a[2] - b[2])
def neg(a): return (-a[0], -a[1], -a[2])
def mul(a, s): return (a[0] * s, a[1] * s, a[2] * s)
def div(a, s): return (a[0] / s, a[1] / s, a[2] / s)
def dot(a, b): return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]
def length(a): return np.sqrt(dot(a, a))
def normalize(a): return mul(a, F(1) / np.sqrt(dot(a, a)))
def cross(a, b): return (a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1])


def m4v(m, v, w):
    """column-major 16 floats times (v, w), glm order"""
    return tuple((m[r] * v[0] + m[4 + r] * v[1]) + (m[8 + r] * v[2] + m[12 + r] * w) for r in range(3))


def m4m4(a, b):
    out = [F(0)] * 16
    for j in range(4):
        for r in range(4):
            s = a[r] * b[4 * j] + a[4 + r] * b[4 * j + 1]
            s = s + a[8 + r] * b[4 * j + 2]
            out[4 * j + r] = s + a[12 + r] * b[4 * j + 3]
    return out


_C = [F(c) for c in (0.16666666666666666, 0.075, 0.044642857142857144, 0.030381944444444444,
                     0.022372159090909092, 0.017352764423076924, 0.01396484375, 0.011551800896139705,
                     0.009761609529194078, 0.008390335809616815, 0.0073125258735988454)]


def _asin(t):
    z = t * t
    p = _C[10]
    for c in reversed(_C[:10]):
        p = p * z + c
    return t + t * (z * p)


def acos(x):
    hi, lo = F(1.57079637050628662109375), F(-4.37113900018624283e-8)
    if x >= F(0.5):
        return F(2) * _asin(np.sqrt((F(1) - x) * F(0.5)))
    if x <= F(-0.5):
        return ((hi - _asin(np.sqrt((F(1) + x) * F(0.5)))) + lo) * F(2)
    return (hi - _asin(x)) + lo


def hash_coords(x, y, z, table):
    h = ((x * 92837111) & 0xFFFFFFFF) ^ ((y * 689287499) & 0xFFFFFFFF) ^ ((z * 283923481) & 0xFFFFFFFF)
    if h >= 1 << 31:
        h -= 1 << 32
    return abs(h) % table


class Scene:
    """One solver holding one or more grid cloths (merged as AddCloth merges them: one
    hash, the last cloth's diameter), with their constraints and the colliders.

    cloths: list of (verts, indices, model (column-major 16), diameter, res, attached),
    registered in order, each followed by its constraint generation."""

    def __init__(self, cloths, colliders, params):
        self.P = params  # dict of floats / ints
        self.x, self.v, self.p, self.w, self.tri = [], [], [], [], []
        self.stretch, self.slots, self.attach, self.bend = [], [], [], []
        self.colliders = colliders
        for verts, indices, model_cm, diameter, res, attached in cloths:
            self._add_cloth(verts, indices, model_cm, diameter, res, attached)
        self.nbr = [[] for _ in range(len(self.x))]

    def _add_cloth(self, verts, indices, model_cm, diameter, res, attached):
        # AddCloth (VtClothSolverGPU.hpp:114-156)
        off = len(self.x)
        pos = [m4v(model_cm, tuple(F(c) for c in v), F(1)) for v in verts]
        n = len(pos)
        self.x += pos
        self.v += [ZERO] * n
        self.p += [ZERO] * n
        self.w += [F(1)] * n
        local_tri = [int(i) for i in indices]
        self.tri += [i + off for i in local_tri]
        self.diameter = F(diameter)
        self.max_speed = F(2) * self.diameter / F(self.P["delta_time"]) * F(self.P["num_substeps"])
        self.spacing = self.diameter * F(self.P["hash_cell_size_scalar"])
        self.T = 2 * len(self.x)
        self.x0 = list(self.x)
        # VtClothObjectGPU::GenerateStretch / GenerateAttach / GenerateBending
        V = res + 1
        at = lambda a, b: off + a * V + b  # noqa: E731
        pairs = []
        for a in range(V):
            for b in range(V):
                if b != res:
                    pairs.append((at(a, b), at(a, b + 1)))
                if a != res:
                    pairs.append((at(a, b), at(a + 1, b)))
                if b != res and a != res:
                    pairs.append((at(a, b), at(a + 1, b + 1)))
                    pairs.append((at(a, b + 1), at(a + 1, b)))
        self.stretch += [(i, j, length(sub(self.x[i], self.x[j]))) for i, j in pairs]
        for pid in attached:
            k = len(self.slots)
            self.slots.append(self.x[off + pid])
            for i in range(off, off + n):
                dist = length(sub(self.slots[k], self.x[i]))
                if dist == 0:
                    self.w[i] = F(0)
                self.attach.append((i, k, dist))
        t = local_tri
        for i in range(0, len(t) - 5, 6):
            self.bend.append((t[i] + off, t[i + 5] + off, t[i + 2] + off, t[i + 1] + off, F(0)))

    # ---------------------------------------------------------------- colliders
    def sdf(self, c, t):
        m = F(self.P["collision_margin"])
        if c["type"] == 1:
            off = t[1] - (c["pos"][1] + m)
            return (F(0), -off, F(0)) if off < 0 else ZERO
        if c["type"] == 0:
            r = c["scale"][0] + m
            d = sub(t, c["pos"])
            dist = length(d)
            off = dist - r
            return mul(div(d, dist), -off) if off < 0 else ZERO
        raise NotImplementedError("cube colliders are not restated here")

    def friction(self, corr, rel):
        fr = ZERO
        cl = length(corr)
        fc = F(self.P["friction"])
        if fc > 0 and cl > 0:
            nrm = div(corr, cl)
            tan = sub(rel, mul(nrm, dot(rel, nrm)))
            tl = length(tan)
            mt = cl * fc
            with np.errstate(divide="ignore", invalid="ignore"):
                fr = mul(neg(tan), np.fmin(mt / tl, F(1)))
        return fr

    def collide_sdf(self, pred, pos, dt):
        out = []
        for i in range(len(pred)):
            po, pr = pos[i], pred[i]
            for c in self.colliders:
                corr = self.sdf(c, pr)
                pr = add(pr, corr)
                if dot(corr, corr) > 0:
                    lp = m4v(c["last_inv"], pr, F(1))
                    vel = div(sub(pr, lp), c["dt"])
                    pr = add(pr, self.friction(corr, sub(sub(pr, po), mul(vel, dt))))
            out.append(pr)
        return out

    # ---------------------------------------------------------------- hash
    def rebuild_hash(self):
        n, T, sp = len(self.p), self.T, self.spacing
        coord = lambda q: tuple(int(np.floor(q[k] / sp)) for k in range(3))  # noqa: E731
        keys = [hash_coords(*coord(q), T) for q in self.p]
        order = sorted(range(n), key=lambda i: (keys[i], i))
        first, last = {}, {}
        for t, i in enumerate(order):
            first.setdefault(keys[i], t)
            last[keys[i]] = t + 1
        mn = self.P["max_num_neighbors"]
        sp2, d2 = sp * sp, self.diameter * self.diameter
        for i in range(n):
            ix, iy, iz = coord(self.p[i])
            lst = []
            full = False
            for X in (ix - 1, ix, ix + 1):
                for Y in (iy - 1, iy, iy + 1):
                    for Z in (iz - 1, iz, iz + 1):
                        h = hash_coords(X, Y, Z, T)
                        if full or h not in first:
                            continue
                        for t in range(first[h], min(last[h], first[h] + mn)):
                            j = order[t]
                            a, b = sub(self.p[i], self.p[j]), sub(self.x0[i], self.x0[j])
                            if j != i and dot(a, a) < sp2 and dot(b, b) > d2:
                                lst.append(j)
                                if len(lst) >= mn:
                                    full = True
                                    break
            self.nbr[i] = lst

    # ---------------------------------------------------------------- constraints
    def apply(self, deltas, counts):
        relax = F(self.P["relaxation_factor"])
        for i in range(len(self.p)):
            if counts[i] > 0:
                self.p[i] = add(self.p[i], mul(div(deltas[i], F(counts[i])), relax))

    def collide_particles(self):
        n = len(self.p)
        deltas, counts = [ZERO] * n, [0] * n
        diam = self.diameter
        for i in range(n):
            d_i, c_i = ZERO, 0
            vi = sub(self.p[i], self.x[i])
            for j in self.nbr[i]:
                den = self.w[i] + self.w[j]
                if den <= 0:
                    continue
                diff = sub(self.p[i], self.p[j])
                dist = length(diff)
                if dist >= diam:
                    continue
                common = mul(div(diff, dist + EPS), (dist - diam) / den)
                c_i += 1
                d_i = sub(d_i, mul(common, self.w[i]))
                rel = sub(vi, sub(self.p[j], self.x[j]))
                d_i = add(d_i, mul(self.friction(common, rel), self.w[i]))
            deltas[i], counts[i] = d_i, c_i
        self.apply(deltas, counts)

    def iteration(self, dt):
        n = len(self.p)
        deltas, counts = [ZERO] * n, [0] * n

        def put(i, c):
            deltas[i] = add(deltas[i], c)
            counts[i] += 1

        for i, j, rest in self.stretch:
            diff = sub(self.p[i], self.p[j])
            d = length(diff)
            if d != rest and self.w[i] + self.w[j] > 0:
                common = mul(div(diff, d + EPS), (d - rest) / (self.w[i] + self.w[j]))
                put(i, mul(common, -self.w[i]))
                put(j, mul(common, self.w[j]))
        lrs = F(self.P["long_range_stretchiness"])
        for i, k, dist in self.attach:
            target = dist * lrs
            if self.w[i] == 0 and target > 0:
                continue
            diff = sub(self.p[i], self.slots[k])
            d = length(diff)
            if d > target:
                put(i, add(neg(diff), mul(div(diff, d), target)))
        bc = F(self.P["bend_compliance"])
        for i0, i1, i2, i3, rest in self.bend:
            p0, p1, p2, p3 = self.p[i0], self.p[i1], self.p[i2], self.p[i3]
            w = (self.w[i0], self.w[i1], self.w[i2], self.w[i3])
            e = sub(p3, p2)
            el = length(e)
            if el < EPS:
                continue
            inv = F(1) / el
            n1 = cross(sub(p2, p0), sub(p3, p0))
            n1 = div(n1, dot(n1, n1))
            n2 = cross(sub(p3, p1), sub(p2, p1))
            n2 = div(n2, dot(n2, n2))
            d = [mul(n1, el), mul(n2, el),
                 add(mul(n1, dot(sub(p0, p3), e) * inv), mul(n2, dot(sub(p1, p3), e) * inv)),
                 add(mul(n1, dot(sub(p2, p0), e) * inv), mul(n2, dot(sub(p2, p1), e) * inv))]
            n1, n2 = normalize(n1), normalize(n2)
            c = dot(n1, n2)
            c = F(-1) if c < F(-1) else c
            c = F(1) if F(1) < c else c
            phi = acos(c)
            lam = w[0] * dot(d[0], d[0]) + w[1] * dot(d[1], d[1])
            lam = lam + w[2] * dot(d[2], d[2])
            lam = lam + w[3] * dot(d[3], d[3])
            if lam < EPS:
                continue
            lam = (phi - rest) / (lam + bc / dt / dt)
            if dot(cross(n1, n2), e) > F(0):
                lam = -lam
            for k, idx in enumerate((i0, i1, i2, i3)):
                put(idx, mul(d[k], -w[k] * lam))
        self.apply(deltas, counts)

    # ---------------------------------------------------------------- frame
    def frame(self, frame_dt, substeps, iterations):
        dt = F(frame_dt) / F(substeps)
        g = tuple(F(c) for c in self.P["gravity"])
        if self.colliders:
            self.x = self.collide_sdf(self.x, self.x, F(frame_dt))
        for s in range(substeps):
            self.v = [add(v, mul(g, dt)) for v in self.v]
            self.p = [add(x, mul(v, dt)) for x, v in zip(self.x, self.v)]
            if self.P["enable_self_collision"]:
                if s % self.P["interleaved_hash"] == 0:
                    self.rebuild_hash()
                self.collide_particles()
            self.p = self.collide_sdf(self.p, self.x, dt)
            for _ in range(iterations):
                self.iteration(dt)
            damp = F(1) - F(self.P["damping"]) * dt
            for i in range(len(self.p)):
                np_ = self.p[i]
                rv = div(sub(np_, self.x[i]), dt)
                rl = length(rv)
                if rl > self.max_speed:
                    rv = mul(div(rv, rl), self.max_speed)
                    np_ = add(self.x[i], mul(rv, dt))
                self.v[i] = mul(rv, damp)
                self.x[i] = np_

    def normals(self):
        acc = [ZERO] * len(self.x)
        for t in range(0, len(self.tri) - 2, 3):
            a, b, c = self.tri[t:t + 3]
            nn = cross(sub(self.x[b], self.x[a]), sub(self.x[c], self.x[a]))
            for k in (a, b, c):
                acc[k] = add(acc[k], nn)
        return [normalize(q) for q in acc]


def collider_dict(c) -> dict:
    """vt_sdf_collider -> the fields this restatement uses (VelocityAt matrix product)."""
    return {"type": int(c.type), "pos": tuple(F(v) for v in c.position), "scale": tuple(F(v) for v in c.scale),
            "dt": F(c.delta_time),
            "last_inv": m4m4([F(v) for v in c.last_transform], [F(v) for v in c.inv_cur_transform])}


def params_dict(p) -> dict:
    return {k: (list(getattr(p, k)) if k == "gravity" else getattr(p, k)) for k, _ in p._fields_}
