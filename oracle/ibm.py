"""PLES's immersed-boundary pieces around the pressure solve.

Test infrastructure: the oracle of ples_mg_potenziale_ibm and of the stop
test of multi with cell types.  Restates:

* potenziale_ibm (fsrc/potenziale_ibm.f03:37-88): for i, j, k in the
  Fortran loop order, a solid cell (tipo 0) is set to 0 and then to the sum
  of its face neighbours that are IB cells (tipo 1), taken in the order
  i+1, i-1, j+1, j-1, k+1, k-1, divided by their count; with no IB
  neighbour it keeps its old value;
* the max-norm stop test of multi with bodyforce = 1
  (fsrc/multigrid.f03:615-631): max |r| over the cells with tipo >= 2.
"""

from __future__ import annotations

import numpy as np


def potenziale_ibm(tipo, fi):
    """tipo, fi: (jx+2, jy+2, jz+2); returns the new fi (plain loops)."""
    fi = np.array(fi, dtype=np.float64, order="F", copy=True)
    jx, jy, jz = (s - 2 for s in fi.shape)
    offs = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))
    for k in range(1, jz + 1):
        for j in range(1, jy + 1):
            for i in range(1, jx + 1):
                if tipo[i, j, k] != 0:
                    continue
                old = fi[i, j, k]
                s, cnt = 0.0, 0
                for di, dj, dk in offs:
                    if tipo[i + di, j + dj, k + dk] == 1:
                        s = s + fi[i + di, j + dj, k + dk]
                        cnt += 1
                fi[i, j, k] = s / cnt if cnt else old
    return fi


def masked_max(tipo, r):
    """max |r| over cells with tipo >= 2; r is (jx, jy, jz)."""
    t = np.asarray(tipo)[1:-1, 1:-1, 1:-1]
    return float(np.abs(np.asarray(r))[t >= 2].max())
