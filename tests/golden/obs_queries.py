"""Evaluates the queries of test/scripted/assets/test_python_obs.py on in-memory results.

Restates the indexing of the reference's .obs reader (opt/python/spinparser/obs.py):
reference/site/cutoff arguments select the nearest basis site, lattice site and recorded
cutoff (obs.py:109-115, :150-178); component "all" is XX + YY + ZZ, which for an SU(2)
file are the same SU2CorZZ dataset (obs.py:21-22, :138-141); the structure factor is
sum_b sum_s chi_bs cos(k (r_s - r_b)) / n_basis in float32 (obs.py:214-249).
"""
from __future__ import annotations

import numpy as np


def _nearest(candidates, x):
    d = np.linalg.norm(np.asarray(candidates) - np.asarray(x), axis=-1)
    return int(np.argmin(d))


def _correlation(q_cutoff, q_site, q_reference, component, cutoffs, zz, tab):
    b = _nearest(tab.basis_pos, q_reference)
    site_list = tab.site_pos[b]
    sites = site_list if (isinstance(q_site, str) and q_site == "all") else np.atleast_2d(np.asarray(q_site, float))
    sidx = [_nearest(site_list, s) for s in sites]
    if isinstance(q_cutoff, str) and q_cutoff == "all":
        cidx = list(range(len(cutoffs)))
    else:
        cidx = [int(np.argmin(np.abs(cutoffs - c))) for c in q_cutoff]
    data = np.stack([zz[c, b, sidx] for c in cidx]).astype(np.float32)
    if component == "all":
        data = data + data + data
    return data


def evaluate_query(q, cutoffs, zz, tab):
    w = q["what"]
    if w == "basis":
        return tab.basis_pos
    if w == "primitives":
        return tab.lattice_vectors
    if w == "sites":
        return tab.site_pos[_nearest(tab.basis_pos, q["reference"])]
    if w == "correlation":
        return _correlation(q["cutoff"], q["site"], q["reference"], q["component"], cutoffs, zz, tab).reshape(-1)
    if w == "structure_factor":
        k = np.atleast_2d(np.asarray(q["momentum"], float))
        cidx = [int(np.argmin(np.abs(cutoffs - c))) for c in q["cutoff"]]
        out = np.zeros((len(cidx), len(k)), np.float32)
        for b in range(tab.n_basis):
            raw = np.stack([zz[c, b, :] for c in cidx]).astype(np.float32) * 3
            rb = tab.basis_pos[b]
            for ic in range(len(cidx)):
                for ik in range(len(k)):
                    for s in range(tab.n_range):
                        out[ic, ik] += raw[ic, s] * np.cos(np.dot(k[ik], tab.site_pos[b, s] - rb))
        out /= tab.n_basis
        return out.reshape(-1)
    raise ValueError(w)
