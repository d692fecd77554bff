"""Oracle (test infrastructure, never product code): CPU restatement of the
reference's irradiance photon map,
PhotonLTEIntegrator::_ConstructIrradiancePhotonMap and _LookupPhotonIrradiance
(Raytracer/LTEIntegrators/PhotonLTEIntegrator/PhotonLTEIntegrator.cpp:127-245),
on the oracle's photon kd-tree (oracle/skw_oracle.cpp, KDTree.h:428-576).

Double-precision sums are taken in the reference's order (the k-NN heap
order), so the results are bit-identical to the reference's."""
from __future__ import annotations

import math

import numpy as np

MAX_NORMAL_DEVIATION_COS = 0.87   # PhotonLTEIntegrator.cpp:26
LOOKUP = 100                      # LOOKUP_PHOTONS_NUM_FOR_IRRADIANCE (PhotonLTEIntegrator.h:218)


def _lookup(kd, weights_t, dir_t, table, q, qn, paths, max_dist):
    """_LookupPhotonIrradiance (:127-169) for every query: (ext, int) float32."""
    res = kd.knn(q, qn, LOOKUP, max_dist, MAX_NORMAL_DEVIATION_COS)
    nq = q.shape[0]
    ext = np.zeros((nq, 3), np.float32)
    intr = np.zeros((nq, 3), np.float32)
    for i in range(nq):
        found = int(res["count"][i])
        if found == 0:
            continue
        px, py, pz = (float(c) for c in q[i])
        nx, ny, nz = (float(c) for c in qn[i])
        se, si, md2 = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0], 0.0
        for j in range(found):
            t = int(res["idx"][i, j])
            pos = kd.pos[kd.perm[t]]
            dx, dy, dz = float(pos[0]) - px, float(pos[1]) - py, float(pos[2]) - pz
            d2 = dx * dx + dy * dy + dz * dz
            if d2 > md2:
                md2 = d2
            d = table[dir_t[t]]
            acc = se if float(d[0]) * nx + float(d[1]) * ny + float(d[2]) * nz > 0.0 else si
            w = weights_t[t]
            for c in range(3):
                acc[c] += float(w[c])
        if found < LOOKUP or md2 == 0.0:
            md2 = max_dist * max_dist
        else:
            md2 *= found / (found - 0.5)
        inv = 1.0 / (math.pi * paths * md2)
        for c in range(3):
            ext[i, c] = np.float32(se[c] * inv)
            intr[i, c] = np.float32(si[c] * inv)
    return ext, intr


def irradiance_map(oracle, maps, paths, scene_area):
    """maps: [caustic, direct, indirect] structured arrays (skwarka_gb300.photon
    PHOTON_DTYPE) in input order.  Returns the irradiance photons in kd-tree
    order (positions, external, internal, normal ids) and the maximum
    irradiance lookup distance."""
    table = oracle.direction_table()
    kds = [oracle.kdtree(m["position"], m["normal"]) if len(m) else None for m in maps]
    ind, kd_ind = maps[2], kds[2]
    if len(ind) == 0:
        e = np.zeros((0, 3), np.float32)
        return e, e, e, np.zeros(0, np.uint16), math.inf
    ind_t = ind[kd_ind.perm]                       # GetAllPoints(): tree order
    irr = ind_t[::10]
    pos = irr["position"].astype(np.float32)
    nrm = irr["normal"].copy()
    q = pos.astype(np.float64)
    qn = table[nrm]
    n_dir, n_ind = len(maps[1]), len(ind)
    da = scene_area / n_dir if n_dir else 0.0
    ia = scene_area / n_ind if n_ind else 0.0
    dist = [0.0, math.sqrt(da * LOOKUP * (1.0 / math.pi)), math.sqrt(ia * LOOKUP * (1.0 / math.pi))]
    dist[0] = max(dist[1], dist[2])
    ext = np.zeros((len(irr), 3), np.float32)
    intr = np.zeros((len(irr), 3), np.float32)
    for m in range(3):
        if kds[m] is None:
            continue
        mt = maps[m][kds[m].perm]
        e, i = _lookup(kds[m], mt["weight"], mt["incident"], table, q, qn, paths[m], dist[m])
        ext = ext + e   # float32: (caustic + direct) + indirect
        intr = intr + i
    kd_irr = oracle.kdtree(pos, nrm)
    p = kd_irr.perm
    pos_t, ext_t, int_t, nrm_t = pos[p], ext[p], intr[p], nrm[p]
    # every 11th indirect photon to its nearest irradiance photon
    sq = ind_t["position"][::11].astype(np.float64)
    sqn = table[ind_t["normal"][::11]]
    near = kd_irr.nearest(sq, sqn, math.inf, MAX_NORMAL_DEVIATION_COS)
    d2 = np.zeros(len(sq))
    for i, t in enumerate(near):
        if t >= 0:
            d = sq[i] - pos_t[t].astype(np.float64)
            d2[i] = float(d[0]) * float(d[0]) + float(d[1]) * float(d[1]) + float(d[2]) * float(d[2])
    index = 0 if len(d2) <= 1 else max(len(d2) // 1000, 1)
    v = np.sort(d2)[::-1][index]
    return pos_t, ext_t, int_t, nrm_t, (math.inf if v == 0.0 else math.sqrt(v))
