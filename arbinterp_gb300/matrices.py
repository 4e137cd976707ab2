"""The interpolation matrices in closed form.

The reference builds ``A = inv(B) @ D`` numerically (src/ARBInterp/ARBInterp.py:107-175,
726-878).  Here A is assembled from its exact factors:

* 3D: ``A = kron(A1, A1, A1)`` with A1 the Catmull-Rom matrix;
* 4D: ``A = kron(A1, A1, A1, A1) + sum_c (h_{c+1} - h_c) s_c^T`` where h_c is
  the inv(B) column of row 240+c (the tensor product of cubic slope-Hermite
  coefficient vectors) and s_c the mixed fourth-difference stencil of corner
  c, with h_16 = 0.  The second term is what the reference's D matrix adds by
  leaving row 240 empty and shifting rows 241..255 by one corner.
"""
from __future__ import annotations

import numpy as np

A1 = np.array([[0.0, 1.0, 0.0, 0.0],
               [-0.5, 0.0, 0.5, 0.0],
               [1.0, -2.5, 2.0, -0.5],
               [-0.5, 1.5, -1.5, 0.5]])

# coefficient vectors of t - 2 t^2 + t^3 and -t^2 + t^3
_HB = np.array([[0.0, 1.0, -2.0, 1.0],
                [0.0, 0.0, -1.0, 1.0]])


def A3() -> np.ndarray:
    return np.kron(np.kron(A1, A1), A1)


def _kron_list(vs):
    out = vs[-1]
    for v in reversed(vs[:-1]):
        out = np.kron(out, v)
    return out


def A4() -> np.ndarray:
    K = np.kron(np.kron(np.kron(A1, A1), A1), A1)
    h = []
    s = []
    for c in range(16):
        bits = [(c >> a) & 1 for a in range(4)]
        # monomial index ex + 4ey + 16ez + 64et: x fastest -> kron(t, z, y, x)
        h.append(_kron_list([_HB[b] for b in bits]))
        st = []
        for b in bits:
            v = np.zeros(4)
            v[b] = -0.5
            v[b + 2] = 0.5
            st.append(v)
        s.append(_kron_list(st))
    corr = np.zeros((256, 256))
    for c in range(16):
        nxt = h[c + 1] if c < 15 else np.zeros(256)
        corr += np.outer(nxt - h[c], s[c])
    return K + corr
