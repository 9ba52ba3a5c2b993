"""Seeded synthetic ephemerides and particle populations.

The JPL files ASSIST is normally run on (DE440 in the ASCII-derived binary
``.440`` layout, the ``sb441-n16.bsp`` asteroid SPK) are not available, so this
module writes files in exactly those layouts whose contents are Chebyshev fits
to Keplerian orbits drawn from a seed:

* ``write_ascii_ephem`` -- a planets file in the layout read by ASSIST's
  ``assist_ascii_init`` (src/ascii_ephem.c:105-252): constant names at 0x00FC,
  header at 0x0A5C, coefficient layout triples, constant values in record 1 and
  32-day data records from record 2 on, with DE440's per-body coefficient
  counts (1018 doubles per record).
* ``write_spk_asteroids`` -- a NAIF DAF/SPK type-2 file read by
  ``assist_spk_init`` / ``assist_spk_calc`` (src/spk.c:267-481): file record,
  one summary + name record pair, one segment per target (heliocentric,
  centre 10, km), each ending with the INIT/INTLEN/RSIZE/N directory.

Bodies: 8 planets + Pluto (EMB for the Earth-Moon pair) on Keplerian orbits
about the barycentre, the Sun's reflex about it, a geocentric Moon and 16
heliocentric asteroids.  Orbits are generated in
an ecliptic frame and rotated by the obliquity into the equatorial frame the
force model assumes.  Particle populations for the five benchmark workloads are
drawn by ``population``.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

AU_KM = 149597870.7
DAY_S = 86400.0
JD_J2000 = 2451545.0
OBLIQUITY = math.radians(23.439291)

# Gravitational parameters (AU^3/day^2) at solar-system magnitudes.
GMS = 2.9591220828411951e-04
GM_PLANETS = {            # ASCII column name -> GM
    "GM1": 4.9124804503647e-11,
    "GM2": 7.2434523326441e-10,
    "GMB": 8.9970116036316e-10,
    "GM4": 9.5495488297258e-11,
    "GM5": 2.8253458252257e-07,
    "GM6": 8.4597059933762e-08,
    "GM7": 1.2920265649682e-08,
    "GM8": 1.5243573478610e-08,
    "GM9": 2.1750964648933e-12,
}
EMRAT = 81.3005682214972154
J2E, J3E, J4E = 1.0826253900e-3, -2.5324105185e-6, -1.6198975999e-6
J2SUN = 2.1961391516529825e-07
RE_KM = 6378.1366
CLIGHT = 299792.458
ASUN_KM = 696000.0

# (column, semi-major axis AU, GM key) for the heliocentric planets, in the
# .440 column order Mercury, Venus, EMB, Mars, Jupiter, Saturn, Uranus, Neptune, Pluto.
PLANETS = [
    ("MER", 0.387, "GM1"), ("VEN", 0.723, "GM2"), ("EMB", 1.000, "GMB"),
    ("MAR", 1.524, "GM4"), ("JUP", 5.20, "GM5"), ("SAT", 9.54, "GM6"),
    ("URA", 19.2, "GM7"), ("NEP", 30.1, "GM8"), ("PLU", 39.5, "GM9"),
]

# .440 column layout: (ncf, niv, ncm) for the 15 columns
# MER VEN EMB MAR JUP SAT URA NEP PLU LUN SUN NUT LIB MAN TDB (DE440 record = 1018 doubles).
LAYOUT = [(14, 4, 3), (10, 2, 3), (13, 2, 3), (11, 1, 3), (8, 1, 3), (7, 1, 3),
          (6, 1, 3), (6, 1, 3), (6, 1, 3), (13, 8, 3), (11, 2, 3), (10, 4, 2),
          (10, 4, 3), (0, 0, 3), (0, 0, 1)]

# Asteroid numbers (NAIF code = 2000000 + number), in the order of the
# 16-body small-body file ASSIST indexes as bodies 11..26.
ASTEROID_NUMBERS = [107, 1, 65, 511, 15, 31, 52, 10, 704, 7, 3, 2, 16, 87, 88, 4]


def _rot_x(v: np.ndarray, ang: float) -> np.ndarray:
    c, s = math.cos(ang), math.sin(ang)
    out = v.copy()
    out[..., 1] = c * v[..., 1] - s * v[..., 2]
    out[..., 2] = s * v[..., 1] + c * v[..., 2]
    return out


@dataclass
class Kepler:
    """Keplerian elements (ecliptic frame) with the central GM; angles in radians."""
    a: np.ndarray
    e: np.ndarray
    inc: np.ndarray
    node: np.ndarray
    peri: np.ndarray
    m0: np.ndarray
    mu: np.ndarray
    epoch: float = 0.0            # days relative to JD 2451545.0

    def state(self, t: np.ndarray, equatorial: bool = True):
        """Heliocentric (or planetocentric) position [AU] and velocity [AU/day]
        at times t (days relative to J2000).  Broadcasting: elements shape (k,),
        t shape (...,) -> result (..., k, 3)."""
        # The mean anomaly n*(t-epoch) reaches hundreds of radians; forming it
        # and reducing it mod 2*pi in long double keeps ~1e-14 AU of rounding
        # noise out of the function the Chebyshev records are fitted to.
        ld = np.longdouble
        t = np.asarray(t, dtype=np.float64)
        n = np.sqrt(self.mu / self.a ** 3)
        n_ld = np.sqrt(self.mu.astype(ld) / self.a.astype(ld) ** 3)
        m = self.m0.astype(ld) + n_ld * (t[..., None].astype(ld) - ld(self.epoch))
        m = np.fmod(m, ld(8) * np.arctan(ld(1))).astype(np.float64)
        e = self.e
        ecc = m + e * np.sin(m)
        for _ in range(60):
            f = ecc - e * np.sin(ecc) - m
            d = f / (1.0 - e * np.cos(ecc))
            ecc = ecc - d
            if np.max(np.abs(d)) < 1e-16:
                break
        ce, se = np.cos(ecc), np.sin(ecc)
        b = self.a * np.sqrt(1.0 - e * e)
        xp = self.a * (ce - e)
        yp = b * se
        edot = n / (1.0 - e * ce)
        vxp = -self.a * se * edot
        vyp = b * ce * edot
        cw, sw = np.cos(self.peri), np.sin(self.peri)
        cn, sn = np.cos(self.node), np.sin(self.node)
        ci, si = np.cos(self.inc), np.sin(self.inc)
        r11 = cn * cw - sn * sw * ci
        r12 = -cn * sw - sn * cw * ci
        r21 = sn * cw + cn * sw * ci
        r22 = -sn * sw + cn * cw * ci
        r31 = sw * si
        r32 = cw * si
        pos = np.stack([r11 * xp + r12 * yp, r21 * xp + r22 * yp, r31 * xp + r32 * yp], axis=-1)
        vel = np.stack([r11 * vxp + r12 * vyp, r21 * vxp + r22 * vyp, r31 * vxp + r32 * vyp], axis=-1)
        if equatorial:
            pos = _rot_x(pos, OBLIQUITY)
            vel = _rot_x(vel, OBLIQUITY)
        return pos, vel


def _draw_elements(rng, a, e_max_deg, i_max_deg, mu):
    k = len(a)
    return Kepler(a=np.asarray(a, float),
                  e=rng.uniform(0.0, e_max_deg, k),
                  inc=np.radians(rng.uniform(0.0, i_max_deg, k)),
                  node=rng.uniform(0, 2 * np.pi, k),
                  peri=rng.uniform(0, 2 * np.pi, k),
                  m0=rng.uniform(0, 2 * np.pi, k),
                  mu=np.asarray(mu, float))


@dataclass
class SolarSystem:
    """Analytic model behind the synthetic files (positions in AU, barycentric)."""
    seed: int
    planets: Kepler = field(init=False)
    moon: Kepler = field(init=False)
    asteroids: Kepler = field(init=False)
    gm_asteroids: np.ndarray = field(init=False)

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        a = [p[1] for p in PLANETS]
        gms = np.array([GM_PLANETS[p[2]] for p in PLANETS])
        self.planets = _draw_elements(rng, a, 0.1, 7.0, GMS + gms)
        # Moon about the Earth, a = 0.00257 AU, e = 0.055
        self.moon = Kepler(a=np.array([0.00257]), e=np.array([0.055]),
                           inc=np.radians(np.array([5.145])),
                           node=rng.uniform(0, 2 * np.pi, 1), peri=rng.uniform(0, 2 * np.pi, 1),
                           m0=rng.uniform(0, 2 * np.pi, 1), mu=np.array([GM_PLANETS["GMB"]]))
        self.gm_asteroids = np.exp(rng.uniform(np.log(1e-14), np.log(1.4e-13), 16))
        self.asteroids = _draw_elements(rng, rng.uniform(2.2, 3.2, 16), 0.2, 15.0, GMS + self.gm_asteroids)
        self.gm_planets = gms

    # --- barycentric states -------------------------------------------------
    def helio_planets(self, t):
        """Barycentric states of the nine planetary bodies (Keplerian about the
        barycentre, which keeps their motion free of the solar reflex)."""
        return self.planets.state(t)

    def sun(self, t):
        """Sun barycentric position/velocity: the reflex that keeps the
        barycentre of the Sun and the nine planetary bodies at the origin."""
        p, v = self.helio_planets(t)
        w = self.gm_planets / GMS
        return -(p * w[:, None]).sum(-2), -(v * w[:, None]).sum(-2)

    def moon_geo(self, t):
        p, v = self.moon.state(t)
        return p[..., 0, :], v[..., 0, :]

    def body(self, idx: int, t):
        """Barycentric pos/vel of ASSIST body index idx (0..26) at times t."""
        t = np.asarray(t, float)
        sp, sv = self.sun(t)
        if idx == 0:
            return sp, sv
        if idx >= 11:
            p, v = self.asteroids.state(t)
            return sp + p[..., idx - 11, :], sv + v[..., idx - 11, :]
        hp, hv = self.helio_planets(t)
        col = {1: 0, 2: 1, 5: 3, 6: 4, 7: 5, 8: 6, 9: 7, 10: 8}
        if idx in col:
            return hp[..., col[idx], :], hv[..., col[idx], :]
        emb_p, emb_v = hp[..., 2, :], hv[..., 2, :]
        mp, mv = self.moon_geo(t)
        if idx == 3:   # Earth = EMB - Moon/(1+EMRAT)
            return emb_p - mp / (1.0 + EMRAT), emb_v - mv / (1.0 + EMRAT)
        return emb_p + mp * (EMRAT / (1.0 + EMRAT)), emb_v + mv * (EMRAT / (1.0 + EMRAT))

    def column_km(self, col: int, t):
        """Value of .440 column `col` (position, km) at times t."""
        t = np.asarray(t, float)
        if col == 10:  # Sun
            return self.sun(t)[0] * AU_KM
        if col == 9:   # geocentric Moon
            return self.moon_geo(t)[0] * AU_KM
        if col <= 8:
            hp, _ = self.helio_planets(t)
            return hp[..., col, :] * AU_KM
        if col == 11:  # nutations: two smooth angles (radians), unused by the force model
            return np.stack([1e-4 * np.sin(t / 6798.4), 4e-5 * np.cos(t / 6798.4)], axis=-1)
        if col == 12:  # librations: three smooth angles
            return np.stack([1e-3 * np.sin(t / 27.3), 4e-4 * np.cos(t / 27.3), 0.4 + 0.23 * t / 27.3], axis=-1)
        raise ValueError(col)


def cheb_fit(func, t_a: np.ndarray, t_b: np.ndarray, ncf: int) -> np.ndarray:
    """Chebyshev interpolation coefficients of func on each [t_a, t_b]:
    returns (k, ncomp, ncf) with f(t) ~= sum_j c_j T_j(tau), tau in [-1,1]."""
    k = np.arange(ncf)
    tau = np.cos(np.pi * (k + 0.5) / ncf)
    mid = 0.5 * (t_a + t_b)
    half = 0.5 * (t_b - t_a)
    ts = mid[:, None] + half[:, None] * tau[None, :]
    vals = func(ts)                                  # (nint, ncf, ncomp)
    tj = np.cos(np.pi * np.outer(np.arange(ncf), k + 0.5) / ncf)   # (ncf, ncf) T_j(tau_k)
    c = (2.0 / ncf) * np.einsum("jk,ikm->imj", tj, vals)
    c[..., 0] *= 0.5
    return c


def _name6(s: str) -> bytes:
    b = s.encode("ascii")
    assert len(b) <= 6
    return b + b" " * (6 - len(b))


def ascii_constants(system: SolarSystem):
    """Ordered (name, value) list written to the constants record."""
    cons = [("DENUM", 440.0), ("LENUM", 440.0), ("TDATEF", 0.0), ("TDATEB", 0.0),
            ("JDEPOC", 2440400.5), ("CENTER", 0.0), ("CLIGHT", CLIGHT), ("BETA", 1.0), ("GAMMA", 1.0),
            ("AU", AU_KM), ("EMRAT", EMRAT), ("GMS", GMS)]
    for _, _, key in PLANETS:
        cons.append((key, GM_PLANETS[key]))
    cons += [("J2E", J2E), ("J3E", J3E), ("J4E", J4E), ("J2SUN", J2SUN), ("RE", RE_KM), ("ASUN", ASUN_KM)]
    for num, gm in zip(ASTEROID_NUMBERS, system.gm_asteroids):
        cons.append(("MA%04d" % num, float(gm)))
    # ASSIST's reader stores the first 400 names unconditionally
    # (src/ascii_ephem.c:159-166), as real DE files (several hundred constants)
    # allow; pad with inert constants so the table holds more than 400 and the
    # names beyond 400 (read from 0x0B28) are exercised too.
    k = 0
    while len(cons) < 420:
        k += 1
        cons.append(("ZZ%04d" % k, 0.0))
    return cons


def write_ascii_ephem(path: str, system: SolarSystem, jd_beg: float, n_rec: int, inc: float = 32.0) -> dict:
    """Write a planets file in the .440 layout covering n_rec records of `inc` days."""
    ncol = len(LAYOUT)
    ndbl = 2 + sum(ncf * niv * ncm for ncf, niv, ncm in LAYOUT)
    rec_bytes = 8 * ndbl
    offs, o = [], 3
    for ncf, niv, ncm in LAYOUT:
        offs.append(o)
        o += ncf * niv * ncm
    cons = ascii_constants(system)
    jd_end = jd_beg + n_rec * inc
    hdr = bytearray(rec_bytes)
    title = [b"JPL Planetary Ephemeris DE440/LE440 (synthetic Keplerian fit)",
             b"Start Epoch: JED=%10.1f" % jd_beg, b"Final Epoch: JED=%10.1f" % jd_end]
    for i, line in enumerate(title):
        hdr[84 * i:84 * i + len(line)] = line
        hdr[84 * i + len(line):84 * (i + 1)] = b" " * (84 - len(line))
    for i, (name, _) in enumerate(cons[:400]):
        hdr[0xFC + 6 * i:0xFC + 6 * i + 6] = _name6(name)
    h = struct.pack("<dddi", jd_beg, jd_end, inc, len(cons)) + struct.pack("<dd", AU_KM, EMRAT)
    for p in range(12):
        h += struct.pack("<iii", offs[p], LAYOUT[p][0], LAYOUT[p][1])
    h += struct.pack("<i", 440) + struct.pack("<iii", offs[12], LAYOUT[12][0], LAYOUT[12][1])
    hdr[0xA5C:0xA5C + len(h)] = h
    assert 0xA5C + len(h) == 0xB28
    tail = b"".join(_name6(name) for name, _ in cons[400:])
    tail += struct.pack("<iiiiii", offs[13], LAYOUT[13][0], LAYOUT[13][1], offs[14], LAYOUT[14][0], LAYOUT[14][1])
    hdr[0xB28:0xB28 + len(tail)] = tail
    conrec = bytearray(rec_bytes)
    vals = np.array([v for _, v in cons], dtype="<f8").tobytes()
    conrec[:len(vals)] = vals

    data = np.zeros((n_rec, ndbl), dtype=np.float64)
    r0 = jd_beg + inc * np.arange(n_rec)
    data[:, 0] = r0
    data[:, 1] = r0 + inc
    for col in range(ncol):
        ncf, niv, ncm = LAYOUT[col]
        if ncf == 0:
            continue
        sub = inc / niv
        ta = (r0[:, None] + sub * np.arange(niv)[None, :]).ravel() - JD_J2000
        c = cheb_fit(lambda t: system.column_km(col, t), ta, ta + sub, ncf)   # (n_rec*niv, ncm, ncf)
        c = c.reshape(n_rec, niv * ncm * ncf)
        data[:, offs[col] - 1: offs[col] - 1 + niv * ncm * ncf] = c
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(bytes(conrec))
        f.write(data.astype("<f8").tobytes())
    return {"jd_beg": jd_beg, "jd_end": jd_end, "inc": inc, "rec_doubles": ndbl, "n_rec": n_rec}


def write_spk_asteroids(path: str, system: SolarSystem, jd_beg: float, jd_end: float,
                        intlen_days: float = 32.0, ncoef: int = 10) -> dict:
    """Write a DAF/SPK type-2 file with one heliocentric segment per asteroid."""
    n_int = int(math.ceil((jd_end - jd_beg) / intlen_days - 1e-12))
    init = (jd_beg - JD_J2000) * DAY_S
    intlen = intlen_days * DAY_S
    rsize = 2 + 3 * ncoef
    seg_len = n_int * rsize + 4
    nt = len(ASTEROID_NUMBERS)
    fward = 2
    data_start_addr = (fward + 1) * 128 + 1          # first double address after summary + name records
    summaries, segments = [], []
    addr = data_start_addr
    ta = jd_beg - JD_J2000 + intlen_days * np.arange(n_int)
    for k, num in enumerate(ASTEROID_NUMBERS):
        def f(t, k=k):
            p, _ = system.asteroids.state(t)
            return p[..., k, :] * AU_KM
        c = cheb_fit(f, ta, ta + intlen_days, ncoef)             # (n_int, 3, ncoef)
        recs = np.zeros((n_int, rsize))
        recs[:, 0] = init + intlen * (np.arange(n_int) + 0.5)
        recs[:, 1] = 0.5 * intlen
        recs[:, 2:] = c.reshape(n_int, 3 * ncoef)
        seg = np.concatenate([recs.ravel(), [init, intlen, float(rsize), float(n_int)]])
        one, two = addr, addr + seg_len - 1
        summaries.append((init, init + n_int * intlen, 2000000 + num, 10, 1, 2, one, two))
        segments.append(seg)
        addr = two + 1
    assert nt <= 25
    filerec = bytearray(1024)
    filerec[0:8] = b"DAF/SPK "
    filerec[8:16] = struct.pack("<ii", 2, 6)
    name = b"synthetic small-body SPK (Keplerian Chebyshev fit)"
    filerec[16:76] = name + b" " * (60 - len(name))
    filerec[76:88] = struct.pack("<iii", fward, fward, addr)
    filerec[88:96] = b"LTL-IEEE"
    sumrec = bytearray(1024)
    sumrec[0:24] = struct.pack("<ddd", 0.0, 0.0, float(nt))
    for i, s in enumerate(summaries):
        sumrec[24 + 40 * i: 24 + 40 * (i + 1)] = struct.pack("<dd6i", *s)
    namerec = bytearray(b" " * 1024)
    for i, s in enumerate(summaries):
        nm = b"AST %d" % s[2]
        namerec[40 * i:40 * i + len(nm)] = nm
    blob = np.concatenate(segments).astype("<f8").tobytes()
    pad = (-len(blob)) % 1024
    with open(path, "wb") as f_:
        f_.write(bytes(filerec))
        f_.write(bytes(sumrec))
        f_.write(bytes(namerec))
        f_.write(blob + b"\0" * pad)
    return {"jd_beg": jd_beg, "jd_end": init / DAY_S + JD_J2000 + n_int * intlen_days, "n_int": n_int,
            "ncoef": ncoef}


def _spk_comment_records(lines) -> list:
    """DAF comment records: lines end with NUL, the area with EOT.  A record
    that ends inside the text ends with one blank so that readers which strip
    each record's trailing NULs (src/spk.c:49-110) do not join two lines."""
    recs, cur = [], b""
    for ln in lines:
        item = ln.encode("ascii") + b"\0"
        if len(cur) + len(item) > 998:
            recs.append(cur + b" ")
            cur = b""
        cur += item
    recs.append(cur + b"\4")
    return [r + b"\0" * (1024 - len(r)) for r in recs]


def write_spk_planets(path: str, system: SolarSystem, jd_beg: float, jd_end: float,
                      intlen_days: float = 16.0, ncoef: int = 12) -> dict:
    """Write the planets as a DAF/SPK type-2 file in the layout of the JPL
    planetary SPK kernels ASSIST reads (src/spk.c, src/assist.c:252-292):
    planet barycentres 1, 2, 4..9, the Sun 10 and the Earth-Moon barycentre 3
    about the solar-system barycentre 0; the Moon 301 and the Earth 399 about
    the Earth-Moon barycentre.  The comment area carries the integration
    constants and GMs ASSIST parses ("KEY value" lines after "Initial
    conditions and constants used for integration:", D exponents)."""
    col = {1: 0, 2: 1, 4: 3, 5: 4, 6: 5, 7: 6, 8: 7, 9: 8}
    fm = EMRAT / (1.0 + EMRAT)
    targets = []
    for code in (1, 2, 3, 4, 5, 6, 7, 8, 9, 10):
        if code == 10:
            targets.append((10, 0, lambda t: system.sun(t)[0] * AU_KM))
        elif code == 3:
            targets.append((3, 0, lambda t: system.helio_planets(t)[0][..., 2, :] * AU_KM))
        else:
            targets.append((code, 0, lambda t, c=col[code]: system.helio_planets(t)[0][..., c, :] * AU_KM))
    targets.append((301, 3, lambda t: system.moon_geo(t)[0] * fm * AU_KM))
    targets.append((399, 3, lambda t: -system.moon_geo(t)[0] / (1.0 + EMRAT) * AU_KM))
    lines = ["Synthetic planetary ephemeris (Keplerian Chebyshev fits).", " ",
             "Initial conditions and constants used for integration:", " "]
    d = lambda v: ("%.17E" % v).replace("E", "D")
    cons = [("AU", AU_KM), ("EMRAT", EMRAT), ("J2E", J2E), ("J3E", J3E), ("J4E", J4E), ("J2SUN", J2SUN),
            ("RE", RE_KM), ("CLIGHT", CLIGHT), ("ASUN", ASUN_KM), ("GMS", GMS)]
    cons += [(key, GM_PLANETS[key]) for _, _, key in PLANETS]
    cons += [("MA%04d" % num, float(gm)) for num, gm in zip(ASTEROID_NUMBERS, system.gm_asteroids)]
    lines += ["%-8s %s" % (k, d(v)) for k, v in cons]
    crecs = _spk_comment_records(lines)
    fward = 2 + len(crecs)
    addr = (fward + 1) * 128 + 1
    summaries, segments = [], []
    for code, cen, f in targets:
        # shorter records for the Moon and the Earth about the Earth-Moon
        # barycentre and for Mercury, as the JPL kernels have
        ilen_d = intlen_days / 4.0 if code in (301, 399) else (intlen_days / 2.0 if code == 1 else intlen_days)
        n_int = int(math.ceil((jd_end - jd_beg) / ilen_d - 1e-12))
        init = (jd_beg - JD_J2000) * DAY_S
        intlen = ilen_d * DAY_S
        rsize = 2 + 3 * ncoef
        seg_len = n_int * rsize + 4
        ta = jd_beg - JD_J2000 + ilen_d * np.arange(n_int)
        c = cheb_fit(f, ta, ta + ilen_d, ncoef)
        recs = np.zeros((n_int, rsize))
        recs[:, 0] = init + intlen * (np.arange(n_int) + 0.5)
        recs[:, 1] = 0.5 * intlen
        recs[:, 2:] = c.reshape(n_int, 3 * ncoef)
        seg = np.concatenate([recs.ravel(), [init, intlen, float(rsize), float(n_int)]])
        one, two = addr, addr + seg_len - 1
        summaries.append((init, init + n_int * intlen, code, cen, 1, 2, one, two))
        segments.append(seg)
        addr = two + 1
    filerec = bytearray(1024)
    filerec[0:8] = b"DAF/SPK "
    filerec[8:16] = struct.pack("<ii", 2, 6)
    name = b"synthetic planetary SPK (Keplerian Chebyshev fit)"
    filerec[16:76] = name + b" " * (60 - len(name))
    filerec[76:88] = struct.pack("<iii", fward, fward, addr)
    filerec[88:96] = b"LTL-IEEE"
    sumrec = bytearray(1024)
    sumrec[0:24] = struct.pack("<ddd", 0.0, 0.0, float(len(summaries)))
    for i, s_ in enumerate(summaries):
        sumrec[24 + 40 * i: 24 + 40 * (i + 1)] = struct.pack("<dd6i", *s_)
    namerec = bytearray(b" " * 1024)
    for i, s_ in enumerate(summaries):
        nm = b"BODY %d" % s_[2]
        namerec[40 * i:40 * i + len(nm)] = nm
    blob = np.concatenate(segments).astype("<f8").tobytes()
    pad = (-len(blob)) % 1024
    with open(path, "wb") as f_:
        f_.write(bytes(filerec))
        for r in crecs:
            f_.write(r)
        f_.write(bytes(sumrec))
        f_.write(bytes(namerec))
        f_.write(blob + b"\0" * pad)
    return {"jd_beg": jd_beg, "jd_end": jd_end, "ncoef": ncoef}


def write_ephemeris(dirpath: str, seed: int = 20240611, t_beg: float = 7800.0, t_end: float = 12000.0):
    """Write planets (.440 layout) + asteroids (SPK) covering [t_beg, t_end]
    (days relative to JD 2451545.0).  Returns (planets_path, asteroids_path, system)."""
    import os
    system = SolarSystem(seed)
    inc = 32.0
    jd0 = JD_J2000 + inc * math.floor(t_beg / inc)
    n_rec = int(math.ceil((JD_J2000 + t_end - jd0) / inc))
    pl = os.path.join(dirpath, "synthetic_%d.440" % seed)
    ast = os.path.join(dirpath, "synthetic_%d_sb16.bsp" % seed)
    write_ascii_ephem(pl, system, jd0, n_rec, inc)
    write_spk_asteroids(ast, system, jd0 - inc, jd0 + (n_rec + 1) * inc)
    return pl, ast, system


def write_planets_spk(dirpath: str, system: SolarSystem, seed: int, t_beg: float, t_end: float) -> str:
    """The same planets as an SPK file (16-day records) covering [t_beg, t_end]."""
    import os
    inc = 32.0
    jd0 = JD_J2000 + inc * math.floor(t_beg / inc)
    n_rec = int(math.ceil((JD_J2000 + t_end - jd0) / inc))
    path = os.path.join(dirpath, "synthetic_%d_planets.bsp" % seed)
    write_spk_planets(path, system, jd0, jd0 + n_rec * inc)
    return path


# ---------------------------------------------------------------------------
# Particle populations (barycentric states at t0, AU and AU/day)
# ---------------------------------------------------------------------------

def _helio_elements(rng, n, kind):
    if kind == "mba":
        a = rng.uniform(2.1, 3.3, n); e = rng.uniform(0.0, 0.3, n); inc = rng.uniform(0, 20, n)
    elif kind == "neo":
        q = rng.uniform(0.9, 1.3, n); e = rng.uniform(0.1, 0.6, n); a = q / (1 - e); inc = rng.uniform(0, 30, n)
    elif kind == "trojan":
        a = rng.uniform(5.05, 5.35, n); e = rng.uniform(0.0, 0.15, n); inc = rng.uniform(0, 30, n)
    elif kind == "tno":
        a = rng.uniform(30, 50, n); e = rng.uniform(0.0, 0.25, n); inc = rng.uniform(0, 30, n)
    else:
        raise ValueError(kind)
    return Kepler(a=a, e=e, inc=np.radians(inc), node=rng.uniform(0, 2 * np.pi, n),
                  peri=rng.uniform(0, 2 * np.pi, n), m0=rng.uniform(0, 2 * np.pi, n),
                  mu=np.full(n, GMS))


def helio_to_bary(system: SolarSystem, t0: float, pos, vel):
    sp, sv = system.sun(np.array(t0))
    return pos + sp, vel + sv


@dataclass
class Population:
    t0: np.ndarray           # (n,) start times, days rel. JD 2451545.0
    t_end: np.ndarray        # (n,)
    state: np.ndarray        # (n, 6) barycentric x,y,z,vx,vy,vz
    params: np.ndarray       # (n, 3) A1, A2, A3
    kind: np.ndarray         # (n,) population label


def population(system: SolarSystem, kind: str, n: int, seed: int, t0: float = 8000.0,
               length: float | None = None, log_len=(30.0, 3652.5), nongrav_frac: float = 0.0,
               close_frac: float = 0.0) -> Population:
    """Draw n particles.  kind: 'mba', 'neo', 'trojan', 'tno' or 'mix' (40/30/20/10).
    length=None draws integration lengths ~ logU[log_len]."""
    rng = np.random.default_rng(seed)
    if kind == "mix":
        kinds = rng.choice(np.array(["mba", "neo", "trojan", "tno"]), size=n, p=[0.4, 0.3, 0.2, 0.1])
    else:
        kinds = np.full(n, kind)
    pos = np.zeros((n, 3)); vel = np.zeros((n, 3))
    for k in np.unique(kinds):
        idx = np.nonzero(kinds == k)[0]
        el = _helio_elements(rng, len(idx), str(k))
        p, v = el.state(np.array(t0))
        pos[idx], vel[idx] = p, v
    pos, vel = helio_to_bary(system, t0, pos, vel)
    if close_frac > 0:
        m = int(round(close_frac * n))
        idx = rng.choice(n, size=m, replace=False)
        ep, ev = system.body(3, np.array(t0))
        d = np.exp(rng.uniform(np.log(1e-4), np.log(1e-2), m))
        u = rng.normal(size=(m, 3)); u /= np.linalg.norm(u, axis=1, keepdims=True)
        w = rng.normal(size=(m, 3)); w -= (w * u).sum(1, keepdims=True) * u
        w /= np.linalg.norm(w, axis=1, keepdims=True)
        vrel = rng.uniform(0.003, 0.012, m)       # 5-20 km/s
        pos[idx] = ep + d[:, None] * u
        vel[idx] = ev + vrel[:, None] * w
        kinds[idx] = "close"
    t0a = np.full(n, float(t0))
    if length is None:
        lens = np.exp(rng.uniform(np.log(log_len[0]), np.log(log_len[1]), n))
    else:
        lens = np.full(n, float(length))
    params = np.zeros((n, 3))
    if nongrav_frac > 0:
        m = int(round(nongrav_frac * n))
        idx = rng.choice(n, size=m, replace=False)
        mag = np.exp(rng.uniform(np.log(1e-12), np.log(1e-9), (m, 2)))
        sgn = rng.choice([-1.0, 1.0], size=(m, 2))
        params[idx, 0:2] = mag * sgn
    return Population(t0=t0a, t_end=t0a + lens, state=np.concatenate([pos, vel], 1), params=params, kind=kinds)
