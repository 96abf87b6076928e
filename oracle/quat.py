"""Oracle: rotation matrix -> unit quaternion (test infrastructure only).

The reference calls ``pyquaternion.Quaternion(matrix=R)`` (camera_approx.py:178;
pyquaternion 0.9.5 pinned in requirements.txt, not installed here) and stores
``q[0..3]`` = (w, x, y, z).  This restates that library's published source,
``Quaternion._from_matrix`` in pyquaternion/quaternion.py: after checking that R is
orthogonal with determinant +1 (``np.allclose``/``np.isclose``, else ValueError), it
returns ``trace_method(R)``, which applies M. Day's branch-on-diagonal method
("Converting a Rotation Matrix to a Quaternion", 2015) to m = R^T (the method assumes
row vectors): the branch is chosen by the sign of m[2,2] and then by comparing m[0,0]
with m[1,1] (or with -m[1,1]); the branch's pivot component is t = 1 +- the diagonal
entries, the others are sums/differences of off-diagonal pairs, and all four are scaled
by 0.5 / sqrt(t).  The constructor does not normalise again.

The sign convention follows from that: the branch's pivot component (w when
m[2,2] >= 0 and m[0,0] >= -m[1,1]) is +0.5 sqrt(t) > 0.
"""
import math

import numpy as np


def quaternion_from_rotation(R):
    m = np.asarray(R, dtype=np.float64).T
    if m[2, 2] < 0:
        if m[0, 0] > m[1, 1]:
            t = 1 + m[0, 0] - m[1, 1] - m[2, 2]
            q = [m[1, 2] - m[2, 1], t, m[0, 1] + m[1, 0], m[2, 0] + m[0, 2]]
        else:
            t = 1 - m[0, 0] + m[1, 1] - m[2, 2]
            q = [m[2, 0] - m[0, 2], m[0, 1] + m[1, 0], t, m[1, 2] + m[2, 1]]
    else:
        if m[0, 0] < -m[1, 1]:
            t = 1 - m[0, 0] - m[1, 1] + m[2, 2]
            q = [m[0, 1] - m[1, 0], m[2, 0] + m[0, 2], m[1, 2] + m[2, 1], t]
        else:
            t = 1 + m[0, 0] + m[1, 1] + m[2, 2]
            q = [t, m[1, 2] - m[2, 1], m[2, 0] - m[0, 2], m[0, 1] - m[1, 0]]
    return np.array(q, dtype=np.float64) * (0.5 / math.sqrt(t))
