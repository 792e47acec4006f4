"""Periodic 2-D tori and the reference's term lists.

The reference reads a ``key=value`` text file (read_input_file.cpp:110-430,
``ED_2D_Lattice_Geometry``) and turns it into three term lists:

* ``adj_list``  -- bonds ``(x, y, J, expphase)``; ``Pairs1`` entries carry J1 and
  ``e^{i phase}`` (read_input_file.cpp:193-214), ``Pairs2`` entries carry J2 and
  phase 1 (:221-240);
* ``ch_list``   -- three cyclic entries ``(i,j,k), (j,k,i), (k,i,j)`` per triangle,
  each with the phase of bond i-j looked up in ``adj_list`` (:249-279, :3-14);
* ``chch_list`` -- "bowtie" entries built from every ordered pair of distinct
  triangles that share a bond endpoint (:286-319).

plus the translation permutations ``T1``/``T2`` (:321-354).

This module builds square and triangular tori with row-major site labels
``s = x + Lx*y`` (T1 = +x, T2 = +y), writes them in the reference's input
format, and parses that format back into the same lists, so the GPU sector,
the oracle and the reference all see identical Hamiltonians.
"""
from __future__ import annotations

import cmath
import dataclasses
import re
from typing import List, Optional, Sequence, Tuple


@dataclasses.dataclass
class Bond:
    """One ``coordinates`` entry (global.h:25-30)."""
    x: int
    y: int
    J: float
    expphase: complex = 1.0 + 0.0j


@dataclasses.dataclass
class Triangle:
    """One ``triangles`` entry (global.h:32-35): bond i-j, Sz part on k."""
    i: int
    j: int
    k: int
    expphase: complex = 1.0 + 0.0j


@dataclasses.dataclass
class Bowtie:
    """One ``bowties`` entry (global.h:37-40)."""
    x: int
    y: int
    z: int
    p: int
    q: int
    r: int


@dataclasses.dataclass
class Model:
    """Everything ``sector_lanczos`` receives (Lanczos_sector.h:11-31)."""
    n_sites: int
    T1: List[int]
    T2: List[int]
    adj_list: List[Bond]
    ch_list: List[Triangle]
    chch_list: List[Bowtie]
    Jz: float = 1.0          # "lambda" in the reference
    J1: float = 1.0
    J2: float = 0.0
    Ch: float = 0.0
    ChCh: float = 0.0
    Sz: float = 0.0
    kx: int = 0
    ky: int = 0
    num_eigenvalues: int = 2
    find_vectors: bool = False
    unwrap_pvector: bool = True
    vector_file_path: str = ""
    tol: float = 1e-11
    lanczos_iterations: int = 100
    lanczos_ncycles: int = 10
    # Not part of the reference file format: the torus the model came from.
    lattice: Optional[str] = None
    Lx: int = 0
    Ly: int = 0
    # 3-D tori (ED_3D_Lattice_Geometry, read_input_file.cpp:443-780): the third
    # translation and its momentum; T3 empty for 2-D models.
    T3: List[int] = dataclasses.field(default_factory=list)
    kz: int = 0
    Lz: int = 1

    @property
    def n_ones(self) -> int:
        """Number of up spins for ``Sz`` (Lanczos_sector.cpp:45-46)."""
        return int(self.Sz + self.n_sites // 2 + 1.0e-6)

    def with_sector(self, Sz: float, kx: int, ky: int, kz: int = 0) -> "Model":
        return dataclasses.replace(self, Sz=float(Sz), kx=int(kx), ky=int(ky), kz=int(kz))


# ----------------------------------------------------------------------------
# torus geometry
# ----------------------------------------------------------------------------

def _site(x: int, y: int, Lx: int, Ly: int) -> int:
    return (x % Lx) + Lx * (y % Ly)


def _bond_set(Lx: int, Ly: int, vectors: Sequence[Tuple[int, int]]) -> List[Tuple[int, int]]:
    seen = set()
    out = []
    for y in range(Ly):
        for x in range(Lx):
            for dx, dy in vectors:
                a = _site(x, y, Lx, Ly)
                b = _site(x + dx, y + dy, Lx, Ly)
                if a == b:
                    raise ValueError(f"bond vector {(dx, dy)} wraps onto itself on {Lx}x{Ly}")
                key = (min(a, b), max(a, b))
                if key in seen:
                    raise ValueError(f"bond vector {(dx, dy)} double-counts bond {key} on {Lx}x{Ly}")
                seen.add(key)
                out.append((a, b))
    return out


SQUARE_NN = [(1, 0), (0, 1)]
SQUARE_NNN = [(1, 1), (1, -1)]
# Triangular lattice in row-major labels: a1 = (1,0), a2 = (0,1) with a2 at 60
# degrees; nearest neighbours along a1, a2 and a2-a1.
TRIANGULAR_NN = [(1, 0), (0, 1), (-1, 1)]
# Next-nearest neighbours (distance sqrt(3)): a1+a2, 2a2-a1, 2a1-a2.
TRIANGULAR_NNN = [(1, 1), (-1, 2), (2, -1)]


def translations(Lx: int, Ly: int) -> Tuple[List[int], List[int]]:
    """T1 = +x, T2 = +y for row-major labels."""
    T1 = [_site(s % Lx + 1, s // Lx, Lx, Ly) for s in range(Lx * Ly)]
    T2 = [_site(s % Lx, s // Lx + 1, Lx, Ly) for s in range(Lx * Ly)]
    return T1, T2


def triangles_ccw(Lx: int, Ly: int) -> List[Tuple[int, int, int]]:
    """Counter-clockwise up and down triangles of the triangular torus.

    up:   (x,y), (x+1,y), (x,y+1)
    down: (x+1,y), (x+1,y+1), (x,y+1)
    """
    out = []
    for y in range(Ly):
        for x in range(Lx):
            out.append((_site(x, y, Lx, Ly), _site(x + 1, y, Lx, Ly), _site(x, y + 1, Lx, Ly)))
            out.append((_site(x + 1, y, Lx, Ly), _site(x + 1, y + 1, Lx, Ly), _site(x, y + 1, Lx, Ly)))
    return out


def _site3(x: int, y: int, z: int, Lx: int, Ly: int, Lz: int) -> int:
    return (x % Lx) + Lx * ((y % Ly) + Ly * (z % Lz))


def translations3(Lx: int, Ly: int, Lz: int) -> Tuple[List[int], List[int], List[int]]:
    """T1 = +x, T2 = +y, T3 = +z for labels s = x + Lx (y + Ly z)."""
    n = Lx * Ly * Lz
    xyz = [(s % Lx, (s // Lx) % Ly, s // (Lx * Ly)) for s in range(n)]
    T1 = [_site3(x + 1, y, z, Lx, Ly, Lz) for x, y, z in xyz]
    T2 = [_site3(x, y + 1, z, Lx, Ly, Lz) for x, y, z in xyz]
    T3 = [_site3(x, y, z + 1, Lx, Ly, Lz) for x, y, z in xyz]
    return T1, T2, T3


def cubic_pairs(Lx: int, Ly: int, Lz: int) -> List[Tuple[int, int]]:
    """Nearest-neighbour bonds of the simple-cubic torus, each listed once
    (along a direction of length 2 the +1 and -1 neighbours coincide)."""
    seen, out = set(), []
    for z in range(Lz):
        for y in range(Ly):
            for x in range(Lx):
                a = _site3(x, y, z, Lx, Ly, Lz)
                for dx, dy, dz in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
                    b = _site3(x + dx, y + dy, z + dz, Lx, Ly, Lz)
                    key = (min(a, b), max(a, b))
                    if a != b and key not in seen:
                        seen.add(key)
                        out.append((a, b))
    return out


def cubic_triangles(Lx: int, Ly: int, Lz: int) -> List[Tuple[int, int, int]]:
    """Triangles (x,y,z), (x+1,y,z), (x,y+1,z) in every xy plane, for the
    chirality term of the cubic torus."""
    return [(_site3(x, y, z, Lx, Ly, Lz), _site3(x + 1, y, z, Lx, Ly, Lz), _site3(x, y + 1, z, Lx, Ly, Lz))
            for z in range(Lz) for y in range(Ly) for x in range(Lx)]


@dataclasses.dataclass
class TorusSpec:
    """A torus plus couplings, before it is turned into reference term lists."""
    lattice: str                 # "square" | "triangular"
    Lx: int
    Ly: int
    Jz: float = 1.0              # Delta (the reference's lambda)
    J1: float = 1.0
    J2: float = 0.0
    Ch: float = 0.0
    ChCh: float = 0.0
    bond_phases: Optional[Sequence[float]] = None   # one phase per Pairs1 entry
    relabel: Optional[Sequence[int]] = None         # optional site permutation
    Lz: int = 1                  # "cubic" only: the third dimension

    @property
    def n_sites(self) -> int:
        return self.Lx * self.Ly * self.Lz

    def pairs1(self):
        if self.lattice == "cubic":
            return cubic_pairs(self.Lx, self.Ly, self.Lz)
        vec = SQUARE_NN if self.lattice == "square" else TRIANGULAR_NN
        return _bond_set(self.Lx, self.Ly, vec)

    def pairs2(self):
        if self.J2 == 0.0:
            return []
        if self.lattice == "cubic":
            raise ValueError("J2 is not defined for the cubic torus")
        vec = SQUARE_NNN if self.lattice == "square" else TRIANGULAR_NNN
        return _bond_set(self.Lx, self.Ly, vec)

    def triangles(self):
        if self.Ch == 0.0 and self.ChCh == 0.0:
            return []
        if self.lattice == "cubic":
            return cubic_triangles(self.Lx, self.Ly, self.Lz)
        if self.lattice != "triangular":
            return []
        return triangles_ccw(self.Lx, self.Ly)


def input_file_text(spec: TorusSpec, Sz: float = 0.0, kx: int = 0, ky: int = 0, *,
                    num_eigenvalues: int = 4, tol: float = 1e-12, iterations: int = 200,
                    ncycles: int = 2, find_vectors: bool = False, kz: int = 0) -> str:
    """Render ``spec`` in the reference's input format (read_input_file.cpp).

    Each key sits on its own line: ``J1=`` does not clear the parser's token
    buffer (read_input_file.cpp:190-191), and ``J1=`` has to precede
    ``Pairs1=`` because J is bound at parse time (:207).  ``Triangles=`` comes
    last because the bowtie list is rebuilt after every character read once
    triangles exist (:286-319).
    """
    perm = list(spec.relabel) if spec.relabel is not None else list(range(spec.n_sites))
    if sorted(perm) != list(range(spec.n_sites)):
        raise ValueError("relabel must be a permutation of the sites")
    cubic = spec.lattice == "cubic"
    if cubic:
        T1, T2, T3 = translations3(spec.Lx, spec.Ly, spec.Lz)
    else:
        T1, T2 = translations(spec.Lx, spec.Ly)
    # new label of old site s is perm[s]; T'[perm[s]] = perm[T[s]]
    T1p = [0] * spec.n_sites
    T2p = [0] * spec.n_sites
    for s in range(spec.n_sites):
        T1p[perm[s]] = perm[T1[s]]
        T2p[perm[s]] = perm[T2[s]]
    p1 = spec.pairs1()
    phases = [float(p) for p in spec.bond_phases] if spec.bond_phases is not None else [0.0] * len(p1)
    if len(phases) != len(p1):
        raise ValueError("one bond phase per Pairs1 entry")
    dims = f"{spec.Lx}x{spec.Ly}" + (f"x{spec.Lz}" if cubic else "")
    lines = [f"[{spec.lattice} torus {dims}, row-major labels]"]
    lines.append(f"tol={tol!r}")
    lines.append(f"Lanczos_iterations={iterations}")
    lines.append(f"Lanczos_ncycles={ncycles}")
    lines.append(f"Jz={spec.Jz!r}")
    lines.append(f"J1={spec.J1!r}")
    lines.append("Pairs1=[" + ",".join(f"[{perm[a]},{perm[b]},{ph!r}]" for (a, b), ph in zip(p1, phases)) + "]")
    p2 = spec.pairs2()
    lines.append(f"J2={spec.J2!r}")
    if p2:
        lines.append("Pairs2=[" + ",".join(f"[{perm[a]},{perm[b]}]" for a, b in p2) + "]")
    lines.append(f"Ch={spec.Ch!r}")
    lines.append(f"ChCh={spec.ChCh!r}")
    lines.append("T1=[" + ",".join(str(t) for t in T1p) + "]")
    lines.append("T2=[" + ",".join(str(t) for t in T2p) + "]")
    if cubic:
        T3p = [0] * spec.n_sites
        for s in range(spec.n_sites):
            T3p[perm[s]] = perm[T3[s]]
        lines.append("T3=[" + ",".join(str(t) for t in T3p) + "]")
    lines.append("Specific_pSector=1")
    lines.append(f"Sz={Sz!r}")
    lines.append(f"kx={kx}")
    lines.append(f"ky={ky}")
    if cubic:
        lines.append(f"kz={kz}")
    lines.append(f"Num_Eigenvalues={num_eigenvalues}")
    lines.append(f"Find_Vectors={int(find_vectors)}")
    tris = spec.triangles()
    if tris:
        lines.append("Triangles=[" + ",".join(f"[{perm[a]},{perm[b]},{perm[c]}]" for a, b, c in tris) + "]")
    return "\n".join(lines) + "\n"


# ----------------------------------------------------------------------------
# parser for the reference input format
# ----------------------------------------------------------------------------

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _expphase_of(i: int, j: int, adj: Sequence[Bond]) -> complex:
    """Phase of bond i-j as seen from i (read_input_file.cpp:3-14)."""
    for b in adj:
        if b.x == i and b.y == j:
            return b.expphase
        if b.x == j and b.y == i:
            return b.expphase.conjugate()
    return 1.0 + 0.0j


def _tri_neighbours(t1: Triangle, t2: Triangle, adj: Sequence[Bond]) -> bool:
    """Two triangles are neighbours when a bond joins any vertex pair
    (read_input_file.cpp:16-45)."""
    a = (t1.i, t1.j, t1.k)
    b = (t2.i, t2.j, t2.k)
    for bd in adj:
        if (bd.x in a and bd.y in b) or (bd.y in a and bd.x in b):
            return True
    return False


def bowties_from_triangles(tris: Sequence[Triangle], adj: Sequence[Bond]) -> List[Bowtie]:
    """Nine bowtie entries per ordered neighbouring triangle pair, in the
    order of read_input_file.cpp:287-318."""
    out: List[Bowtie] = []
    for m, t1 in enumerate(tris):
        for n, t2 in enumerate(tris):
            if m == n or not _tri_neighbours(t1, t2, adj):
                continue
            firsts = [(t1.i, t1.j, t1.k), (t1.k, t1.i, t1.j), (t1.j, t1.k, t1.i)]
            seconds = [(t2.i, t2.j, t2.k), (t2.k, t2.i, t2.j), (t2.j, t2.k, t2.i)]
            for (x, y, z) in firsts:
                for (p, q, r) in seconds:
                    out.append(Bowtie(x, y, z, p, q, r))
    return out


def parse_input_text(text: str, bowties: bool = True) -> Model:
    """Parse the reference input format into a :class:`Model`.

    Follows routine_parameters (read_input_file.cpp:59-108) and
    ED_2D_Lattice_Geometry (:110-430): lines whose first non-blank character
    is ``[`` are comments, J1/J2 are bound to pairs at the time the pair list
    is read, every triangle expands into three cyclic ``ch_list`` entries.
    """
    vals = dict(Jz=1.0, J1=1.0, J2=0.0, Ch=0.0, ChCh=0.0)
    adj: List[Bond] = []
    ch: List[Triangle] = []
    tri_first: List[Triangle] = []
    T1: List[int] = []
    T2: List[int] = []
    T3: List[int] = []
    kw = {}
    for raw in text.splitlines():
        line = "".join(raw.split())
        if not line or line.startswith("["):
            continue
        key, _, rest = line.partition("=")
        if key in ("Jz", "J1", "J2", "Ch", "ChCh"):
            vals[key] = float(re.match(_NUM, rest).group(0))
        elif key == "Pairs1":
            for a, b, ph in re.findall(rf"\[(-?\d+),(-?\d+),({_NUM})\]", rest):
                adj.append(Bond(int(a), int(b), vals["J1"], cmath.exp(1j * float(ph))))
        elif key == "Pairs2":
            for a, b in re.findall(r"\[(-?\d+),(-?\d+)\]", rest):
                adj.append(Bond(int(a), int(b), vals["J2"], 1.0 + 0.0j))
        elif key == "Triangles":
            for a, b, c in re.findall(r"\[(-?\d+),(-?\d+),(-?\d+)\]", rest):
                x, y, z = int(a), int(b), int(c)
                t1 = Triangle(x, y, z, _expphase_of(x, y, adj))
                t2 = Triangle(y, z, x, _expphase_of(y, z, adj))
                t3 = Triangle(z, x, y, _expphase_of(z, x, adj))
                tri_first.append(t1)
                ch.extend([t1, t2, t3])
        elif key in ("T1", "T2", "T3"):
            nums = [int(n) for n in re.findall(r"-?\d+", rest)]
            {"T1": T1, "T2": T2, "T3": T3}[key].extend(nums)
        elif key in ("Sz",):
            kw["Sz"] = float(re.match(_NUM, rest).group(0))
        elif key in ("kx", "ky", "kz", "Num_Eigenvalues", "Lanczos_iterations", "Lanczos_ncycles"):
            kw[key] = int(re.match(r"-?\d+", rest).group(0))
        elif key in ("Find_Vectors", "Unwrap_pVector"):
            kw[key] = bool(int(re.match(r"-?\d+", rest).group(0)))
        elif key == "tol":
            kw["tol"] = float(re.match(_NUM, rest).group(0))
        elif key == "Vector_File_Path":
            kw["Vector_File_Path"] = rest
    if len(T1) != len(T2):
        raise ValueError("ERROR: input T1 != T2")   # read_input_file.cpp:423-427
    if T3 and len(T3) != len(T1):
        raise ValueError("ERROR: input T1 != T2 != T3")   # read_input_file.cpp:774-778
    chch = bowties_from_triangles(tri_first, adj) if (tri_first and bowties) else []
    return Model(
        n_sites=len(T1), T1=T1, T2=T2, adj_list=adj, ch_list=ch, chch_list=chch,
        Jz=vals["Jz"], J1=vals["J1"], J2=vals["J2"], Ch=vals["Ch"], ChCh=vals["ChCh"],
        Sz=kw.get("Sz", -1.0), kx=kw.get("kx", -1), ky=kw.get("ky", -1),
        num_eigenvalues=kw.get("Num_Eigenvalues", 2), find_vectors=kw.get("Find_Vectors", False),
        unwrap_pvector=kw.get("Unwrap_pVector", True), vector_file_path=kw.get("Vector_File_Path", ""),
        tol=kw.get("tol", 1e-11), lanczos_iterations=kw.get("Lanczos_iterations", 100),
        lanczos_ncycles=kw.get("Lanczos_ncycles", 10), T3=T3, kz=kw.get("kz", 0),
    )


def make_model(spec: TorusSpec, Sz: float = 0.0, kx: int = 0, ky: int = 0, bowties: bool = True, **kw) -> Model:
    """Build the term lists for ``spec`` exactly as the reference parser would.
    ``bowties=False`` leaves the ChCh bowtie list empty (it is O(triangles^2)
    to build and unused when ChCh is 0)."""
    m = parse_input_text(input_file_text(spec, Sz, kx, ky, **kw), bowties=bowties)
    m.lattice, m.Lx, m.Ly, m.Lz = spec.lattice, spec.Lx, spec.Ly, spec.Lz
    return m
