"""Readers and writers for the CRMod/CRTomo input and output files.

The formats are the reference's, parsed with Fortran list-directed read
semantics (one READ statement consumes as many records as it needs and
discards the rest of its last record):

* ``elem.dat``  -- src/relem.f90:7-326 (and cutmckee/relem.f, welem.f)
* ``elec.dat``  -- src/relectr.f90:7-89 (cutmckee/welectr.f)
* ``rho.dat``   -- src/rsigma.f90:8-260
* ``config.dat``-- src/rdatm.f90:6-136
* ``crmod.cfg`` -- src/fem.f90:163-205
* ``volt.dat``  -- src/wdatm.f90 (written by CRMod)
* boundary values -- src/rrandb.f90 (lrandb2)
* potentials and sensitivities -- src/wpot.f90, src/wsens.f90 (one file per
  measurement)

Node, element and electrode numbers are kept 1-based, exactly as in the
files, so that the arrays can be handed to the C ABI unchanged.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import List, Optional, Sequence

import numpy as np

from . import fortran_io as FIO


class CRError(RuntimeError):
    """Error carrying one of the reference's error numbers (src/error.txt)."""

    def __init__(self, errnr: int, text: str = ""):
        super().__init__(f"errnr {errnr}: {text}")
        self.errnr = errnr
        self.text = text


# ---------------------------------------------------------------------------
# list-directed record reader
# ---------------------------------------------------------------------------
class _Records:
    def __init__(self, path: str):
        self.path = path
        with open(path, "r") as fh:
            self.lines = fh.read().splitlines()
        self.pos = 0

    @staticmethod
    def _tokens(line: str) -> List[str]:
        out = []
        for tok in line.replace(",", " ").replace("\t", " ").split():
            if tok.startswith("!"):
                break
            if tok == "/":
                break
            out.append(tok)
        return out

    def read(self, n: int) -> List[str]:
        """One list-directed READ of n items."""
        vals: List[str] = []
        while len(vals) < n:
            if self.pos >= len(self.lines):
                raise CRError(2, f"end of file in {self.path}")
            toks = self._tokens(self.lines[self.pos])
            self.pos += 1
            for t in toks:
                if "*" in t and t.split("*")[0].isdigit():
                    r, v = t.split("*", 1)
                    vals.extend([v] * int(r))
                else:
                    vals.append(t)
        return vals[:n]

    def read_line(self) -> str:
        if self.pos >= len(self.lines):
            raise CRError(2, f"end of file in {self.path}")
        s = self.lines[self.pos]
        self.pos += 1
        return s

    def backspace(self):
        self.pos = max(0, self.pos - 1)


def _f(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def _logical(tok: str) -> bool:
    t = tok.strip().lstrip(".").upper()
    if t.startswith("T"):
        return True
    if t.startswith("F"):
        return False
    raise ValueError(tok)


# ---------------------------------------------------------------------------
# grid
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Grid:
    """FE grid (src/elemmod.f90).  Boundary element types (> 10) come last."""

    sanz: int
    mb: int
    typ: np.ndarray      # int32 (typanz)
    nelanz: np.ndarray   # int32 (typanz)
    selanz: np.ndarray   # int32 (typanz)
    snr: np.ndarray      # int32 (sanz), node -> coordinate index, 1-based
    sx: np.ndarray       # float64 (sanz)
    sy: np.ndarray       # float64 (sanz)
    nrel: np.ndarray     # int32 (elanz+relanz, maxnk), 1-based node numbers
    rnr: np.ndarray      # int32 (relanz), boundary -> adjacent element, 1-based

    @property
    def typanz(self) -> int:
        return int(len(self.typ))

    @property
    def elanz(self) -> int:
        return int(sum(n for t, n in zip(self.typ, self.nelanz) if t <= 10))

    @property
    def relanz(self) -> int:
        return int(sum(n for t, n in zip(self.typ, self.nelanz) if t > 10))

    @property
    def maxnk(self) -> int:
        return int(max(self.selanz))

    def node_xy(self):
        """Coordinates in node-number order: x[node-1], y[node-1]."""
        return self.sx[self.snr - 1], self.sy[self.snr - 1]

    def nrel_colmajor(self) -> np.ndarray:
        """nrel in Fortran column-major order (the C ABI layout)."""
        return np.ascontiguousarray(self.nrel.T, dtype=np.int32)

    def copy(self) -> "Grid":
        return dataclasses.replace(
            self, typ=self.typ.copy(), nelanz=self.nelanz.copy(), selanz=self.selanz.copy(),
            snr=self.snr.copy(), sx=self.sx.copy(), sy=self.sy.copy(), nrel=self.nrel.copy(),
            rnr=self.rnr.copy())


def fix_border_elements(grid: Grid) -> int:
    """Border-to-element consistency fix of src/relem.f90:207-237.

    For each boundary element, the reference scans all area elements and sets
    rnr to the LAST element (in element order) whose first selanz(1) nodes
    contain both boundary nodes.  Returns the number of corrections.
    Raises CRError(111) if a pointer stays out of range (relem.f90:239-250).
    """
    elanz, relanz = grid.elanz, grid.relanz
    nk1 = int(grid.selanz[0])
    area = grid.nrel[:elanz, :nk1]
    owners = {}
    for e in range(elanz):
        for node in area[e]:
            owners.setdefault(int(node), []).append(e + 1)
    nfix = 0
    for i in range(relanz):
        ik1, ik2 = int(grid.nrel[elanz + i, 0]), int(grid.nrel[elanz + i, 1])
        cands = set(owners.get(ik1, ())) & set(owners.get(ik2, ()))
        if cands:
            k = max(cands)
            if k != int(grid.rnr[i]):
                # the reference re-assigns at every mismatching match; the
                # final value is the largest matching element
                nfix += 1
                grid.rnr[i] = k
    bad = np.count_nonzero((grid.rnr > elanz) | (grid.rnr < 1))
    if bad:
        raise CRError(111, "border to element context is wrong")
    return nfix


def read_elem(path: str, fix_borders: bool = True) -> Grid:
    """src/relem.f90:7-326."""
    r = _Records(path)
    sanz, typanz, mb = (int(x) for x in r.read(3))
    t = [int(x) for x in r.read(3 * typanz)]
    typ = np.array(t[0::3], np.int32)
    nelanz = np.array(t[1::3], np.int32)
    selanz = np.array(t[2::3], np.int32)
    v = r.read(3 * sanz)
    snr = np.array([int(x) for x in v[0::3]], np.int32)
    sx = np.array([_f(x) for x in v[1::3]], np.float64)
    sy = np.array([_f(x) for x in v[2::3]], np.float64)
    ne = int(nelanz.sum())
    maxnk = int(selanz.max())
    nrel = np.zeros((ne, maxnk), np.int32)
    idum = 0
    for i in range(typanz):
        for j in range(int(nelanz[i])):
            nrel[idum + j, : selanz[i]] = [int(x) for x in r.read(int(selanz[i]))]
        idum += int(nelanz[i])
    relanz = int(sum(n for tt, n in zip(typ, nelanz) if tt > 10))
    rnr = np.array([int(x) for x in r.read(relanz)], np.int32) if relanz else np.zeros(0, np.int32)
    g = Grid(sanz=sanz, mb=mb, typ=typ, nelanz=nelanz, selanz=selanz, snr=snr, sx=sx, sy=sy,
             nrel=nrel, rnr=rnr)
    if fix_borders and relanz:
        fix_border_elements(g)
    return g


def write_elem(path: str, g: Grid):
    """cutmckee/welem.f: list-directed header, nodes as I8,2F12.3 (real*4)."""
    with open(path, "w") as fh:
        fh.write(f"{g.sanz:12d}{g.typanz:12d}{g.mb:12d}\n")
        for t, n, s in zip(g.typ, g.nelanz, g.selanz):
            fh.write(f"{int(t):12d}{int(n):12d}{int(s):12d}\n")
        for i in range(g.sanz):
            fh.write(f"{int(g.snr[i]):8d}{float(np.float32(g.sx[i])):12.3f}"
                     f"{float(np.float32(g.sy[i])):12.3f}\n")
        idum = 0
        for t, n, s in zip(g.typ, g.nelanz, g.selanz):
            for j in range(int(n)):
                fh.write("".join(f"{int(x):12d}" for x in g.nrel[idum + j, :s]) + "\n")
            idum += int(n)
        for x in g.rnr:
            fh.write(f"{int(x):12d}\n")


# ---------------------------------------------------------------------------
# electrodes, measurements, resistivity
# ---------------------------------------------------------------------------
def read_elec(path: str, sanz: Optional[int] = None) -> np.ndarray:
    """src/relectr.f90:7-89 -> enr (int32, 1-based node numbers)."""
    r = _Records(path)
    eanz = int(r.read(1)[0])
    enr = np.array([int(r.read(1)[0]) for _ in range(eanz)], np.int32)
    if sanz is not None and np.any(enr > sanz):
        raise CRError(29, "electrode node beyond sanz")
    return enr


def write_elec(path: str, enr: np.ndarray):
    with open(path, "w") as fh:
        fh.write(f"{len(enr):12d}\n")
        for e in enr:
            fh.write(f"{int(e):12d}\n")


@dataclasses.dataclass
class Survey:
    """Electrodes and four-point configurations (src/electrmod.f90,
    src/datmod.f90).  strnr/vnr use the reference encoding A*10000 + B."""

    enr: np.ndarray     # int32 (eanz)
    strnr: np.ndarray   # int32 (nanz)
    vnr: np.ndarray     # int32 (nanz)
    strom: np.ndarray   # float64 (nanz)

    @property
    def eanz(self) -> int:
        return int(len(self.enr))

    @property
    def nanz(self) -> int:
        return int(len(self.strnr))

    def electrodes(self):
        """(e1, e2, e3, e4) with e1 = mod(strnr,10000) (src/bvolt.f90:44-49)."""
        e1 = self.strnr % 10000
        e2 = (self.strnr - e1) // 10000
        e3 = self.vnr % 10000
        e4 = (self.vnr - e3) // 10000
        return e1, e2, e3, e4


def check_config(strnr, vnr, eanz: int):
    """Electrode checks of src/rdatm.f90:54-81 (errors 46 and 73)."""
    for i, (s, v) in enumerate(zip(strnr, vnr)):
        e1 = s % 10000
        e2 = (s - e1) // 10000
        e3 = v % 10000
        e4 = (v - e3) // 10000
        if min(e1, e2, e3, e4) < 0 or max(e1, e2, e3, e4) > eanz:
            raise CRError(46, f"Electrode pair {i + 1} not correct")
        if (e1 == e2 or e3 == e4 or (((e1 == e3) or (e1 == e4)) and e1 != 0)
                or (((e2 == e3) or (e2 == e4)) and e2 != 0)):
            raise CRError(73, f"duplicate electrodes for reading {i + 1}")


def read_config(path: str, eanz: int):
    """src/rdatm.f90:6-136 -> (strnr, vnr, strom)."""
    r = _Records(path)
    nanz = int(r.read(1)[0])
    first = int(r.read(1)[0])
    r.backspace()
    crtf = first - 10000 >= 0
    strnr = np.zeros(nanz, np.int32)
    vnr = np.zeros(nanz, np.int32)
    for i in range(nanz):
        if crtf:
            a, b = r.read(2)
            strnr[i], vnr[i] = int(a), int(b)
        else:
            e1, e2, e3, e4 = (int(x) for x in r.read(4))
            strnr[i] = e1 * 10000 + e2
            vnr[i] = e3 * 10000 + e4
    check_config(strnr, vnr, eanz)
    return strnr, vnr, np.ones(nanz, np.float64)


def write_config(path: str, strnr, vnr):
    with open(path, "w") as fh:
        fh.write(f"{len(strnr)}\n")
        for s, v in zip(strnr, vnr):
            fh.write(f"{int(s):12d}{int(v):12d}\n")


def read_rho(path: str, elanz: int) -> np.ndarray:
    """src/rsigma.f90:8-260 (no prior, no reference model values).

    Returns sigma (complex128, elanz) = (cos(phi) - i sin(phi)) / |rho| with
    phi in mrad."""
    r = _Records(path)
    first = r._tokens(r.read_line())
    idum = int(first[0])
    if idum != elanz:
        raise CRError(47, "rho.dat element count mismatch")
    lw_ref = False
    if len(first) >= 2:
        try:
            lw_ref = _logical(first[1])
        except ValueError:
            lw_ref = False
    sig = np.zeros(elanz, np.complex128)
    for i in range(elanz):
        vals = r.read(6 if lw_ref else 2)
        bet = _f(vals[0])
        pha = 1e-3 * _f(vals[1])
        if bet < 1e-12:
            raise CRError(11, "resistivity <= 0")
        sig[i] = complex(math.cos(pha) / bet, -math.sin(pha) / bet)
    return sig


def write_rho(path: str, mag: np.ndarray, pha_mrad: np.ndarray):
    with open(path, "w") as fh:
        fh.write(f"{len(mag)}\n")
        for a, p in zip(mag, pha_mrad):
            fh.write(f"{float(a):.9e} {float(p):.9e}\n")


# ---------------------------------------------------------------------------
# crmod.cfg and volt.dat
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class CRModConfig:
    """crmod.cfg (src/fem.f90:163-205)."""

    delem: str
    delectr: str
    dsigma: str
    dstrom: str
    lpot: bool
    dpot: str
    lvolt: bool
    dvolt: str
    lsens: bool
    dsens: str
    lagain: bool
    swrtr: int
    lsink: bool
    nsink: int
    lrandb2: bool
    drandb: str
    mswitch: int = 0

    @property
    def lana(self) -> bool:
        return bool(self.mswitch & 1) and not self.lsr

    @property
    def wkfak(self) -> bool:
        return bool(self.mswitch & 2)

    @property
    def lsr(self) -> bool:
        return bool(self.mswitch & 4)


def read_crmod_cfg(path: str) -> CRModConfig:
    with open(path) as fh:
        lines = fh.read().splitlines()

    def name(s):
        return s[:80].strip()

    def first(s):
        return _Records._tokens(s)[0]

    it = iter(lines)
    next(it)  # header line
    v = {}
    v["delem"] = name(next(it))
    v["delectr"] = name(next(it))
    v["dsigma"] = name(next(it))
    v["dstrom"] = name(next(it))
    v["lpot"] = _logical(first(next(it)))
    v["dpot"] = name(next(it))
    v["lvolt"] = _logical(first(next(it)))
    v["dvolt"] = name(next(it))
    v["lsens"] = _logical(first(next(it)))
    v["dsens"] = name(next(it))
    v["lagain"] = _logical(first(next(it)))
    v["swrtr"] = int(first(next(it)))
    v["lsink"] = _logical(first(next(it)))
    v["nsink"] = int(first(next(it)))
    v["lrandb2"] = _logical(first(next(it)))
    v["drandb"] = name(next(it))
    mswitch = 0
    try:
        s = next(it)
        mswitch = int(s[:4])
    except (StopIteration, ValueError):
        mswitch = 0
    v["mswitch"] = mswitch
    return CRModConfig(**v)


def volt_record(sigmaa: np.ndarray, strnr: np.ndarray, vnr: np.ndarray):
    """Magnitude, phase (mrad) and possibly swapped vnr as src/wdatm.f90:60-76
    computes them (before the real*4 conversion)."""
    bet = np.abs(sigmaa)
    pha = np.arctan2(sigmaa.imag, sigmaa.real)
    npi = np.rint(pha / math.pi) * math.pi
    swap = np.abs(npi) > 1e-12
    pha = np.where(swap, pha - npi, pha)
    ie1 = vnr % 10000
    ie2 = (vnr - ie1) // 10000
    vout = np.where(swap, ie1 * 10000 + ie2, vnr).astype(np.int32)
    return bet, 1e3 * pha, vout


def write_volt(path: str, strnr, vnr, sigmaa):
    """src/wdatm.f90:55-76, byte for byte as gfortran writes it: nanz, then
    strnr, vnr, real(|sigmaa|), real(1e3 phase) list-directed, with the
    voltage electrodes swapped where the phase wraps."""
    bet, pha, vout = volt_record(np.asarray(sigmaa), np.asarray(strnr), np.asarray(vnr))
    with open(path, "w") as fh:
        fh.write(FIO.record([FIO.int4(len(strnr))]))
        for s, v, b, p in zip(strnr, vout, bet, pha):
            fh.write(FIO.record([FIO.int4(s), FIO.int4(v), FIO.real4(b), FIO.real4(p)]))


def read_volt(path: str):
    """volt.dat written by CRMod: (strnr, vnr, magnitude, phase_mrad)."""
    r = _Records(path)
    nanz = int(r.read(1)[0])
    s = np.zeros(nanz, np.int32)
    v = np.zeros(nanz, np.int32)
    bet = np.zeros(nanz)
    pha = np.zeros(nanz)
    for i in range(nanz):
        vals = r.read(4)
        s[i], v[i] = int(vals[0]), int(vals[1])
        bet[i], pha[i] = _f(vals[2]), _f(vals[3])
    return s, v, bet, pha


def _read_items(rec: _Records, kinds: Sequence[str]) -> list:
    """One list-directed READ of integers ("i"), reals ("r") and complex
    numbers ("c", written ``(re, im)``; a bare real reads as re + 0i)."""
    out: list = []
    toks: List[str] = []
    q = 0
    while len(out) < len(kinds):
        if q >= len(toks):
            toks = rec._tokens(rec.read_line())
            q = 0
            continue
        kind = kinds[len(out)]
        t = toks[q]
        if kind == "c" and t.startswith("("):
            parts = [t]
            while not parts[-1].endswith(")"):
                q += 1
                while q >= len(toks):
                    toks = rec._tokens(rec.read_line())
                    q = 0
                parts.append(toks[q])
            nums = " ".join(parts).strip("()").replace("(", " ").replace(")", " ").split()
            if len(nums) != 2:
                raise CRError(3, f"complex value {' '.join(parts)!r} in {rec.path}")
            out.append(complex(_f(nums[0]), _f(nums[1])))
        elif kind == "i":
            out.append(int(t))
        elif kind == "c":
            out.append(complex(_f(t), 0.0))
        else:
            out.append(_f(t))
        q += 1
    return out


def read_boundary_values(path: str, sanz: int):
    """Boundary values of src/rrandb.f90 (complex case): rwdanz, then rwdanz
    records ``node value`` (Dirichlet), then rwnanz and rwnanz values
    (Neumann; read and not used, as in the reference).  Returns (nodes int32
    1-based, values complex128).  A node above sanz raises errnr 30."""
    rec = _Records(path)
    n = _read_items(rec, "i")[0]
    nodes = np.zeros(n, np.int32)
    vals = np.zeros(n, np.complex128)
    for i in range(n):
        nodes[i], vals[i] = _read_items(rec, "ic")
        if nodes[i] > sanz:
            raise CRError(30, f"boundary node {nodes[i]} in {path}")
    nn = _read_items(rec, "i")[0]
    if nn > 0:
        _read_items(rec, "c" * nn)
    return nodes, vals


def write_boundary_values(path: str, nodes, values):
    """The file read by read_boundary_values (no Neumann values)."""
    with open(path, "w") as fh:
        fh.write(f"{len(nodes)}\n")
        for k, v in zip(nodes, values):
            v = complex(v)
            fh.write(f"{int(k)} ({v.real!r},{v.imag!r})\n")
        fh.write("0\n")


def f4(x) -> str:
    """A REAL*4 value as gfortran's list-directed output prints it (9
    significant digits), without the field's padding."""
    return FIO.real4(x).strip()


def numbered_path(datei: str, i: int, count: int) -> str:
    """The file name of measurement i (1-based) of count, as src/wpot.f90 and
    src/wsens.f90 form it: the number, zero-padded to the digits of count,
    before the extension of datei ("pot.dat" -> "pot0001.dat")."""
    head, tail = os.path.split(datei)
    lnanz = int(math.log10(count)) + 1
    stem, dot, ext = tail.partition(".")
    return os.path.join(head, f"{stem}{i:0{lnanz}d}{dot}{ext[:3]}")


def write_potentials(datei: str, hpot: np.ndarray, strnr, strom, grid: "Grid"):
    """src/bpot.f90 + src/wpot.f90: for every measurement the potential of its
    current pair (hpot(e2) - hpot(e1), times strom) at every node, as
    x y Re Im lines, node by node in band order.  hpot: (eanz, sanz)."""
    x, y = grid.node_xy()
    nanz = len(strnr)
    os.makedirs(os.path.dirname(datei) or ".", exist_ok=True)
    for i in range(nanz):
        e1, e2 = int(strnr[i]) % 10000, int(strnr[i]) // 10000
        if e1 == 0:
            pot = hpot[e2 - 1] * strom[i]
        elif e2 == 0:
            pot = -hpot[e1 - 1] * strom[i]
        else:
            pot = (hpot[e2 - 1] - hpot[e1 - 1]) * strom[i]
        with open(numbered_path(datei, i + 1, nanz), "w") as fh:  # src/wpot.f90:82-85
            fh.write("".join(FIO.record([FIO.real4(x[j]), FIO.real4(y[j]), FIO.real4(pot[j].real),
                                         FIO.real4(pot[j].imag)]) for j in range(len(pot))))


def write_sensitivities(datei: str, sens: np.ndarray, cx: np.ndarray, cy: np.ndarray):
    """src/wsens.f90: one file per measurement i: |sum_j J_ij| and its phase
    (mrad), then x y Re Im of J_ij for every element j (centroids cx, cy).
    sens: (nanz, manz)."""
    nanz = sens.shape[0]
    os.makedirs(os.path.dirname(datei) or ".", exist_ok=True)
    for i in range(nanz):
        summe = complex(np.sum(sens[i]))
        with open(numbered_path(datei, i + 1, nanz), "w") as fh:  # src/wsens.f90:82-93
            if abs(summe) > 0.0:
                fh.write(FIO.record([FIO.real4(abs(summe)), FIO.real4(1e3 * math.atan2(summe.imag, summe.real))]))
            else:
                fh.write(FIO.record([FIO.real4(0.0), FIO.real4(0.0)]))
            fh.write("".join(FIO.record([FIO.real4(cx[j]), FIO.real4(cy[j]), FIO.real4(sens[i, j].real),
                                         FIO.real4(sens[i, j].imag)]) for j in range(sens.shape[1])))


@dataclasses.dataclass
class Tomodir:
    """A CRMod working set loaded from crmod.cfg."""

    cfg: CRModConfig
    grid: Grid
    survey: Survey
    sigma: np.ndarray
    boundary_values: Optional[tuple] = None  # (nodes, values) when lrandb2


def load_crmod(exe_dir: str, config_override: Optional[str] = None) -> Tomodir:
    """Load the inputs named by exe_dir/crmod.cfg (src/fem.f90:163-302)."""
    cfg = read_crmod_cfg(os.path.join(exe_dir, "crmod.cfg"))

    def p(x):
        return os.path.normpath(os.path.join(exe_dir, x))

    grid = read_elem(p(cfg.delem))
    enr = read_elec(p(cfg.delectr), grid.sanz)
    cpath = config_override or p(cfg.dstrom)
    strnr, vnr, strom = read_config(cpath, len(enr))
    sigma = read_rho(p(cfg.dsigma), grid.elanz)
    bv = read_boundary_values(p(cfg.drandb), grid.sanz) if cfg.lrandb2 else None
    return Tomodir(cfg=cfg, grid=grid, survey=Survey(enr=enr, strnr=strnr, vnr=vnr, strom=strom),
                   sigma=sigma, boundary_values=bv)
