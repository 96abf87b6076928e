"""Oracle: 3x3 median blur (test infrastructure only).

The reference filters every DSM with ``cv2.medianBlur(img.astype(np.float32), 3)``
(produce_dsm.py:58, aggregate_2p5d.py:81).  OpenCV (4.0.0.21 pinned) is not installed,
so this restates the documented behaviour -- each output pixel is the median of its
3x3 neighbourhood, borders replicated -- and fixes the behaviour OpenCV leaves
undocumented: NaN sorts after every number (numpy's sort order), so the output is
the 5th smallest of the 9 values, which is NaN only when at least 5 of them are NaN.
Parity of this step with OpenCV is unpinned.
"""
import numpy as np


def median_blur3x3(img):
    img = np.asarray(img, dtype=np.float32)
    H, W = img.shape
    pad = np.pad(img, 1, mode='edge')
    stack = np.stack([pad[1 + dj:1 + dj + H, 1 + dk:1 + dk + W]
                      for dj in (-1, 0, 1) for dk in (-1, 0, 1)], axis=0)
    return np.sort(stack, axis=0)[4]
