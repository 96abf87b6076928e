"""Oracle: rotation matrix -> unit quaternion (test infrastructure only).

The reference calls ``pyquaternion.Quaternion(matrix=R)`` (camera_approx.py:178;
pyquaternion 0.9.5, not installed here).  That library converts with the
branch-on-largest-diagonal method of M. Day, "Converting a Rotation Matrix to a
Quaternion" (2015), applied to R^T; this restates that published method.  Parity of
the quaternion's overall sign is unpinned (no reference output is available).
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
