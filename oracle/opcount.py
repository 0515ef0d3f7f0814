"""Operation count of one Wirz push in the ABC field (test infrastructure).

TEST INFRASTRUCTURE ONLY: pins the per-push FP64 work behind the FP64 path's
throughput figures.  A Python restatement of the oracle's or_wirz
(src/tracking.c:749-892) and of the ABC field (getemf_ff / getb_ff,
src/force_free.c:54-66,138-150, no velocity grid, so E = 0) runs on an
operation-counting scalar; tests/test_opcount.py checks that the same
restatement on plain floats reproduces the oracle bit for bit, so the count
belongs to the operations the reference performs.
"""
import math


class Counter:
    def __init__(self):
        self.n = {"add": 0, "mul": 0, "div": 0, "sqrt": 0, "sin": 0, "cos": 0}

    def flops(self):
        """add/sub, mul and div as one operation each (sqrt, sin, cos listed apart)."""
        return self.n["add"] + self.n["mul"] + self.n["div"]


class Num:
    """A float that counts the arithmetic done with it."""
    __slots__ = ("v", "c")

    def __init__(self, v, c):
        self.v = float(v)
        self.c = c

    def _w(self, o):
        return o.v if isinstance(o, Num) else float(o)

    def _op(self, kind, v):
        self.c.n[kind] += 1
        return Num(v, self.c)

    def __add__(self, o): return self._op("add", self.v + self._w(o))
    def __radd__(self, o): return self._op("add", self._w(o) + self.v)
    def __sub__(self, o): return self._op("add", self.v - self._w(o))
    def __rsub__(self, o): return self._op("add", self._w(o) - self.v)
    def __mul__(self, o): return self._op("mul", self.v * self._w(o))
    def __rmul__(self, o): return self._op("mul", self._w(o) * self.v)
    def __truediv__(self, o): return self._op("div", self.v / self._w(o))
    def __rtruediv__(self, o): return self._op("div", self._w(o) / self.v)
    def __neg__(self): return Num(-self.v, self.c)  # sign flip, no arithmetic


def _fn(name, x):
    if isinstance(x, Num):
        x.c.n[name] += 1
        return Num(getattr(math, name)(x.v), x.c)
    return getattr(math, name)(x)


def sqrt(x): return _fn("sqrt", x)
def sin(x): return _fn("sin", x)
def cos(x): return _fn("cos", x)


def abc_field(x, y, z, A, B, C, B0, lam):
    """getb_ff (src/force_free.c:138-150) times B0; E = 0 without a velocity grid."""
    bx = A * sin(lam * z) + C * cos(lam * y)
    by = B * sin(lam * x) + A * cos(lam * z)
    bz = C * sin(lam * y) + B * cos(lam * x)
    return (bx * B0, by * B0, bz * B0), (0.0, 0.0, 0.0)


def wirz(p, dt, cm, field):
    """One push; p = [x, y, z, ux, uy, uz, t], field(x, y, z, t) -> (B, E).
    Same operations and order as or_wirz."""
    x, y, z, ux, uy, uz, t0 = p
    r0 = (x, y, z)
    delta = (ux, uy, uz)
    gama = sqrt(1.0 + delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2])
    B, E = field(x, y, z, t0)
    Btot = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2])
    iBtot = 1.0 / Btot
    dth = dt * 0.5
    dm = [delta[i] + cm * dth * E[i] for i in range(3)]
    gama = sqrt(1.0 + dm[0] * dm[0] + dm[1] * dm[1] + dm[2] * dm[2])
    igama = 1.0 / gama
    vminus = [dm[i] * igama for i in range(3)]
    hpara = [B[i] * iBtot for i in range(3)]
    vdothp = 0.0
    for i in range(3):
        vdothp = vdothp + vminus[i] * hpara[i]
    c = [vminus[i] - vdothp * hpara[i] for i in range(3)]
    vperp = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])
    hperp = [(vminus[i] - vdothp * hpara[i]) / vperp for i in range(3)]
    hr = [hpara[1] * hperp[2] - hpara[2] * hperp[1], hpara[2] * hperp[0] - hpara[0] * hperp[2],
          hpara[0] * hperp[1] - hpara[1] * hperp[0]]
    gyroR = vperp * gama * 1.0 * iBtot / cm
    omegac = cm * Btot * igama
    dtheta = omegac * dt
    sind, cosd = sin(dtheta * 0.5), cos(dtheta * 0.5)
    tmp1, tmp2, tmp3 = dth * vdothp * 1.0, gyroR * sind, -gyroR * (1.0 - cosd)
    pre = [r0[i] + hpara[i] * tmp1 + hperp[i] * tmp2 + hr[i] * tmp3 for i in range(3)]
    B, E = field(pre[0], pre[1], pre[2], t0 + dth)
    Btot = sqrt(B[0] * B[0] + B[1] * B[1] + B[2] * B[2])
    iBtot = 1.0 / Btot
    hpara = [B[i] * iBtot for i in range(3)]
    vdothp = 0.0
    for i in range(3):
        vdothp = vdothp + vminus[i] * hpara[i]
    c = [vminus[i] - vdothp * hpara[i] for i in range(3)]
    vperp = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])
    hperp = [(vminus[i] - vdothp * hpara[i]) / vperp for i in range(3)]
    hr = [hpara[1] * hperp[2] - hpara[2] * hperp[1], hpara[2] * hperp[0] - hpara[0] * hperp[2],
          hpara[0] * hperp[1] - hpara[1] * hperp[0]]
    omegac = cm * Btot * igama
    dtheta = omegac * dt
    sind, cosd = sin(dtheta), cos(dtheta)
    vplus = [hpara[i] * vdothp + vperp * (cosd * hperp[i] - sind * hr[i]) for i in range(3)]
    bm = 0.0
    for i in range(3):
        bm = bm + vplus[i] * vplus[i]
    g2 = 1.0 / sqrt(1.0 - bm)
    delta = [g2 * vplus[i] for i in range(3)]
    u = [delta[i] + cm * dth * E[i] for i in range(3)]
    vdothp = 0.0
    for i in range(3):
        vdothp = vdothp + vplus[i] * hpara[i]
    c = [vplus[i] - vdothp * hpara[i] for i in range(3)]
    vperp = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])
    gyroR = vperp * gama * 1.0 * iBtot / cm
    tmp1, tmp2, tmp3 = dt * vdothp * 1.0, gyroR * sind, -gyroR * (1.0 - cosd)
    xyz = [r0[i] + (hpara[i] * tmp1 + hperp[i] * tmp2 + hr[i] * tmp3) for i in range(3)]
    return [xyz[0], xyz[1], xyz[2], u[0], u[1], u[2], t0 + dt]


def count_abc_push(A=1.0, B=1.0, C=1.0, B0=1.0, lam=2 * math.pi, cm=1.0, dt=0.05):
    """Operation counts of one push and of one field evaluation (ABC, E = 0)."""
    c = Counter()
    p = [Num(v, c) for v in (0.3, 0.6, 0.2, 0.4, -0.5, 0.7, 0.0)]
    wirz(p, dt, cm, lambda x, y, z, t: abc_field(x, y, z, A, B, C, B0, lam))
    cf = Counter()
    q = [Num(v, cf) for v in (0.3, 0.6, 0.2)]
    abc_field(q[0], q[1], q[2], A, B, C, B0, lam)
    return c.n, cf.n
