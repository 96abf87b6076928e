"""Oracle: ``cv2.medianBlur(img.astype(np.float32), 3)`` (test infrastructure only).

The reference filters every DSM with OpenCV's 3x3 median (produce_dsm.py:58,
aggregate_2p5d.py:81; opencv-python 4.0.0.21 pinned in requirements.txt, not installed
here).  This restates OpenCV 4.0.0's own implementation of that call, from its published
source (modules/imgproc/src/median_blur.cpp, ``cv::medianBlur`` ->
``medianBlur_SortNet<MinMax32f, MinMaxVec32f>`` for ksize 3 and CV_32F), so that what
it does with NaN -- which OpenCV does not document -- follows from the code:

* Window: rows i-1, i, i+1 and columns j-1, j, j+1, clamped into the image
  (BORDER_REPLICATE).  p0..p8 are the window row by row.
* Network: the 19 compare-exchanges of the 9-input median network of A. Paeth
  (Graphics Gems, 1990) in N. Devillard's order ("Fast median search: an ANSI C
  implementation", 1998): (1,2) (4,5) (7,8) (0,1) (3,4) (6,7) (1,2) (4,5) (7,8) (0,3)
  (5,8) (4,7) (3,6) (1,4) (2,5) (4,7) (4,2) (6,4) (4,2); the output is p4.
* Compare-exchange op(a, b): OpenCV computes ``t = a; a = min(a, b); b = max(b, t)``.
  - Scalar columns use ``MinMax32f`` (std::min / std::max): ``std::min(a, b)`` is
    ``b < a ? b : a`` and ``std::max(b, t)`` is ``b < t ? t : b``, so the pair is
    exchanged only when b < a; ties and NaN leave it as it is.
  - Vector columns use ``MinMaxVec32f`` on 4-lane SSE registers (``_mm_min_ps``,
    ``_mm_max_ps``), which return their second operand unless the comparison holds:
    ``a = a < b ? a : b`` and ``b = b > t ? b : t``.  The pair stays only when a < b;
    ties (so -0/+0) and NaN exchange it.
* Which columns are vector columns (x86-64, where SSE2 is always present): per row the
  scalar loop runs column 0, the vector loop then runs 4 columns at a time from column 1
  while ``j <= W - 4 - 1``, and the scalar loop finishes the rest.  So columns
  [1, 1 + 4 * nv) with nv = (W - 6) // 4 + 1 for W >= 6 (else none) are vector columns.
* A 1-pixel-high or 1-pixel-wide image takes a separate path: the median of 3 along the
  line (neighbours clamped), op(p0, p1) op(p1, p2) op(p0, p1) with the scalar op,
  output p1.

Pinning: this follows OpenCV's source path.  An OpenCV build may hand the call to a
vendor library instead (Intel IPP, whose code is closed); that route, if the pinned
wheel takes it, cannot be restated.  ``median_blur3x3_loop`` is the same algorithm
written pixel by pixel, checked equal to the vectorised form by the tests.
"""
import numpy as np

# Paeth's 9-input median network in Devillard's order (pairs of window positions).
NETWORK = ((1, 2), (4, 5), (7, 8), (0, 1), (3, 4), (6, 7), (1, 2), (4, 5), (7, 8), (0, 3),
           (5, 8), (4, 7), (3, 6), (1, 4), (2, 5), (4, 7), (4, 2), (6, 4), (4, 2))
SIMD_LANES = 4     # 128-bit SSE registers of float32


def vector_columns(W):
    """Boolean mask over the W columns that OpenCV's 4-lane loop handles."""
    nv = (W - 6) // 4 + 1 if W >= 6 else 0
    mask = np.zeros(W, dtype=bool)
    mask[1:1 + SIMD_LANES * nv] = True
    return mask


def _exchange(a, b, vec):
    """One compare-exchange; ``vec`` selects the SSE op (element-wise)."""
    with np.errstate(invalid='ignore'):
        swap = np.where(vec, ~(a < b), b < a)
    return np.where(swap, b, a), np.where(swap, a, b)


def _median3_line(line):
    """The 1-D path: median of 3 along a line with clamped neighbours, scalar op."""
    n = line.size
    p0 = line[np.maximum(np.arange(n) - 1, 0)]
    p1 = line.copy()
    p2 = line[np.minimum(np.arange(n) + 1, n - 1)]
    no = np.zeros(n, dtype=bool)
    p0, p1 = _exchange(p0, p1, no)
    p1, p2 = _exchange(p1, p2, no)
    p0, p1 = _exchange(p0, p1, no)
    return p1


def median_blur3x3(img):
    img = np.asarray(img, dtype=np.float32)
    H, W = img.shape
    if H == 1 or W == 1:
        return _median3_line(img.ravel()).reshape(H, W).astype(np.float32)
    rows = (np.maximum(np.arange(H) - 1, 0), np.arange(H), np.minimum(np.arange(H) + 1, H - 1))
    cols = (np.maximum(np.arange(W) - 1, 0), np.arange(W), np.minimum(np.arange(W) + 1, W - 1))
    p = [img[r][:, c] for r in rows for c in cols]           # p0..p8, row by row
    vec = np.broadcast_to(vector_columns(W), (H, W))
    for i, j in NETWORK:
        p[i], p[j] = _exchange(p[i], p[j], vec)
    return p[4].astype(np.float32)


def _op_scalar(a, b):
    t = a
    a = b if b < a else a          # std::min(a, b)
    b = t if b < t else b          # std::max(b, t)
    return a, b


def _op_vector(a, b):
    t = a
    a = a if a < b else b          # _mm_min_ps(a, b)
    b = b if b > t else t          # _mm_max_ps(b, t)
    return a, b


def median_blur3x3_loop(img):
    """Pixel-by-pixel form of ``median_blur3x3`` (small images only)."""
    img = np.asarray(img, dtype=np.float32)
    H, W = img.shape
    out = np.empty_like(img)
    if H == 1 or W == 1:
        line = img.ravel()
        n = line.size
        res = np.empty_like(line)
        for i in range(n):
            p0, p1, p2 = line[max(i - 1, 0)], line[i], line[min(i + 1, n - 1)]
            p0, p1 = _op_scalar(p0, p1)
            p1, p2 = _op_scalar(p1, p2)
            p0, p1 = _op_scalar(p0, p1)
            res[i] = p1
        return res.reshape(H, W)
    vec = vector_columns(W)
    for i in range(H):
        r = (max(i - 1, 0), i, min(i + 1, H - 1))
        for j in range(W):
            c = (max(j - 1, 0), j, min(j + 1, W - 1))
            p = [img[rr, cc] for rr in r for cc in c]
            op = _op_vector if vec[j] else _op_scalar
            for a, b in NETWORK:
                p[a], p[b] = op(p[a], p[b])
            out[i, j] = p[4]
    return out
