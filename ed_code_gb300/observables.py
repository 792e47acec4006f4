"""Expectation values of the reference's analysis operators between momentum
eigenvectors, without leaving the momentum basis.

The reference (analysis/src/pspincorr.cpp, pchirality.cpp) unwraps both
eigenvectors into the fixed-Sz basis and sums the operator's matrix elements
there (chirality_exp.cpp: szsz_op, sxsxsysy_op, ch_op).  Here both vectors
stay in their (Sz, kx, ky) sector.  For two states of the same sector the
matrix element of a term O_{ij} equals that of its translation average
(1/|G|) sum_g O_{g(i) g(j)}, because both states pick up the same phase
under every translation.  That average is a Hamiltonian of this library's
own form, with bonds or triangles on the term's orbit and weight 1/|G|, so
one GPU H*v gives the matrix element:
  * SxSx + SySy on (i, j):  <bra| H(bonds of the orbit, Delta = 0) |ket>,
  * SzSz on (i, j):         <bra| H(Delta = 1) - H(Delta = 0) |ket>,
  * the chirality of a triangle list, as pchirality reports it
    (i times the cyclic sum of ch_op): minus <bra| H(chirality terms) |ket>.
Vectors are normalised momentum-basis coefficient arrays (complex128, n_p).
"""
from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import lattice as L
from .sector import GpuSector


def translations(model: L.Model) -> List[List[int]]:
    """Every translation T2^b T1^a (a < L1, b < L2) as a site permutation."""
    T1, T2 = model.T1, model.T2
    L1 = 1
    s = T1[0]
    while s != 0:
        s, L1 = T1[s], L1 + 1
    L2 = 1
    s = T2[0]
    while s != 0:
        s, L2 = T2[s], L2 + 1
    out = []
    for a in range(L1):
        for b in range(L2):
            g = list(range(model.n_sites))
            for _ in range(a):
                g = [T1[x] for x in g]
            for _ in range(b):
                g = [T2[x] for x in g]
            out.append(g)
    return out


def _element(model: L.Model, bra: np.ndarray, ket: np.ndarray, bonds=(), tris=(), Jz: float = 0.0,
             Ch: float = 0.0) -> complex:
    op = dataclasses.replace(model, adj_list=list(bonds), ch_list=list(tris), chch_list=[], Jz=Jz, Ch=Ch, ChCh=0.0,
                             J2=0.0)
    sec = GpuSector(op)
    try:
        if len(ket) != sec.n_p or len(bra) != sec.n_p:
            raise ValueError(f"vectors must have the sector's {sec.n_p} entries")
        return complex(np.vdot(bra, sec.sHv(np.asarray(ket, np.complex128))))
    finally:
        sec.close()


def spin_correlations(model: L.Model, pairs: Sequence[Tuple[int, int]], ket: np.ndarray,
                      bra: Optional[np.ndarray] = None) -> Dict[Tuple[int, int], Dict[str, complex]]:
    """<bra| Sz_i Sz_j |ket> and <bra| SxSx + SySy |ket> for each pair (i, j),
    as szsz_op and sxsxsysy_op define them (bra defaults to ket)."""
    bra = ket if bra is None else bra
    G = translations(model)
    out = {}
    for i, j in pairs:
        bonds = [L.Bond(g[i], g[j], 1.0 / len(G)) for g in G]
        xy = _element(model, bra, ket, bonds=bonds, Jz=0.0)
        full = _element(model, bra, ket, bonds=bonds, Jz=1.0)
        out[(i, j)] = {"SzSz": full - xy, "SxSx+SySy": xy}
    return out


def chirality(model: L.Model, triangles: Sequence[Tuple[int, int, int]], ket: np.ndarray,
              bra: Optional[np.ndarray] = None) -> complex:
    """The chirality expectation pchirality reports for a triangle list: i times
    the sum over the triangles of ch_op(i,j,k) + ch_op(j,k,i) + ch_op(k,i,j)."""
    bra = ket if bra is None else bra
    G = translations(model)
    tris = []
    for (i, j, k) in triangles:
        for g in G:
            a, b, c = g[i], g[j], g[k]
            tris += [L.Triangle(a, b, c), L.Triangle(b, c, a), L.Triangle(c, a, b)]
    return -_element(model, bra, ket, tris=tris, Ch=1.0 / len(G))
