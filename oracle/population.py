"""CPU restatement of the reference's particle deletion and creation (TEST
INFRASTRUCTURE: the checker of libuwg's uwg_pop_* entry points, never the
product).

The swarm is held the way the reference holds it: one particle array
(coordinates, owning cell and every per-particle data column) and one list of
particle indices per cell.  The edits follow the reference line by line:
* Swarm_DeleteParticle (L/StgDomain/Swarm/src/SwarmClass.c:1032-1085) with
  Swarm_RemoveParticleFromCell (:1016-1030): the particle leaves its cell by
  swap-with-last, the array's last particle is copied into its slot and its
  cell entry relabelled;
* EscapedRoutine_RemoveFromSwarm
  (L/PICellerator/PopulationControl/src/EscapedRoutine.c:174-284): particles
  outside the mesh, collected in index order and removed from the highest down;
* _PCDVC_Calculate2D/3D, non-aggressive path (L/PICellerator/Utils/src/PCDVC.c:
  313-700, 703-1084): per cell in order, split the particles whose Voronoi
  volume exceeds upT*vol/100 (the first maxSplits in cell order; the copy goes to
  the end of the array and of the cell, at FeMesh_CoordLocalToGlobal of the
  particle's Voronoi centroid), then delete those below lowT*vol/100 (largest
  index first, at most maxDeletions).
Voronoi volumes and centroids come from the oracle's DVC (``Mesh.pic_map``).
"""
import numpy as np


class RefSwarm:
    def __init__(self, coords, owner, cells, data, n_cells):
        self.x = [np.array(c, dtype=np.float64) for c in coords]
        self.owner = [int(o) for o in owner]
        self.cells = [list(c) for c in cells]
        self.data = {k: [np.array(r) for r in v] for k, v in data.items()}
        self.n_cells = n_cells

    @property
    def n(self):
        return len(self.x)

    def _copy(self, src, dst):
        self.x[dst] = self.x[src].copy()
        self.owner[dst] = self.owner[src]
        for v in self.data.values():
            v[dst] = v[src].copy()

    def _pop_last(self):
        self.x.pop()
        self.owner.pop()
        for v in self.data.values():
            v.pop()

    def _fill_from_last(self, p):
        last = self.n - 1
        if p != last:
            lc = self.owner[last]
            lpos = self.cells[lc].index(last)
            self._copy(last, p)
            self.cells[lc][lpos] = p
        self._pop_last()

    def delete_particle(self, p):
        c = self.owner[p]
        L = self.cells[c]
        pos = L.index(p)
        L[pos] = L[-1]
        L.pop()
        self._fill_from_last(p)

    def remove_escaped(self):
        esc = sorted(p for p in range(self.n) if self.owner[p] >= self.n_cells)
        for p in reversed(esc):
            self._fill_from_last(p)

    def split(self, c, slot, coord):
        src = self.cells[c][slot]
        self.x.append(self.x[src].copy())
        self.owner.append(c)
        for v in self.data.values():
            v.append(v[src].copy())
        new = self.n - 1
        self.x[new] = np.array(coord, dtype=np.float64)
        self.cells[c].append(new)

    def tables(self):
        off = np.zeros(self.n_cells + 1, np.int64)
        off[1:] = np.cumsum([len(c) for c in self.cells])
        lst = np.array([p for c in self.cells for p in c], dtype=np.int64)
        return off, lst


def pcdvc(m, swarm, weights, centroids, id_key, split_threshold, delete_threshold, max_splits, max_deletions):
    """Population control of ``swarm`` (a RefSwarm whose data column ``id_key``
    holds each particle's original index, the index of ``weights``/``centroids``)."""
    upT, lowT = split_threshold * 100., delete_threshold * 100.
    vol = 4 if m.dim == 2 else 8
    maxW, minW = upT * vol / 100.0, lowT * vol / 100.0
    ids = swarm.data[id_key]
    n_split = n_del = 0
    for c in range(swarm.n_cells):
        L = list(swarm.cells[c])
        orig = [int(ids[p][0]) for p in L]
        split_slots = [j for j, o in enumerate(orig) if weights[o] > maxW]
        dels = sorted((p for p, o in zip(L, orig) if weights[o] < minW), reverse=True)
        for j in split_slots[:max_splits]:
            swarm.split(c, j, m.local_to_global(c, centroids[orig[j]]))
            n_split += 1
        for p in dels[:max_deletions]:
            swarm.delete_particle(p)
            n_del += 1
    return n_split, n_del
