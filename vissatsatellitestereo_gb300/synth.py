"""Seeded synthetic workloads for the VisSat geometry path.

The reference runs on WorldView-3 scenes of the MVS3DM benchmark.  None of that data
is available offline, so every input here is drawn from fixed-seed distributions with
the shapes, layouts and value ranges the reference sees:

* RPC cameras shaped like the dictionaries ``lib/parse_meta.py`` produces and
  ``RPCModel.__init__`` consumes (``lib/rpc_model.py:132-158``): ten offsets/scales,
  four 20-term coefficient lists, image width and height.
* lat/lon/alt sample grids laid out exactly like ``gen_grid`` (``lib/gen_grid.py:38-56``,
  z-major, ``ij`` meshgrid inside a slab), with ENU coordinates about the grid centre
  at the lowest altitude as ``coordinate_system.py:45-47`` chooses its origin.
* height maps of a "box city" scene sampled through a per-view pixel->UTM affine map,
  flattened into (easting, northing, height) point lists -- the layout
  ``aggregate_2p5d_util.py:96-98`` hands to ``proj_to_grid``.

Small cases are generated with numpy (bit-reproducible on any host); the large
per-view point clouds use torch so that they can be generated directly in device memory.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .geodesy import geodetic_to_enu

BASE_SEED = 20261203

# Explorer AOI of the MVS3DM benchmark (UTM zone 21 S), used as the UTM anchor so the
# FP64 origin subtraction of the rasteriser sees realistic magnitudes.
EXPLORER_UL_EASTING = 354052.3651180889
EXPLORER_UL_NORTHING = 6182702.10540914


# --------------------------------------------------------------------------------------
# RPC cameras
# --------------------------------------------------------------------------------------
def make_rpc_meta(seed: int, width: int = 2048, height: int = 2048) -> dict:
    """One synthetic RPC camera in the ``meta_dict`` format ``RPCModel`` takes.

    Offsets: LAT_OFF~U(20,50) deg, LONG_OFF~U(-120,120) deg, HEIGHT_OFF~U(0,500) m;
    LAT/LONG_SCALE = 0.05 deg, HEIGHT_SCALE = 500 m; LINE/SAMP_OFF = LINE/SAMP_SCALE =
    half the image size.  The numerator linear terms are +-1 (+N(0,0.05)) on the RPC
    slot of the matching axis (colNum[1] <- lon, rowNum[2] <- lat, north up), every other
    numerator term N(0,1e-3); the denominators are 1 + N(0,1e-4) terms.
    """
    rng = np.random.default_rng(seed)
    col_num = rng.normal(0.0, 1e-3, 20)
    row_num = rng.normal(0.0, 1e-3, 20)
    col_num[1] = 1.0 + rng.normal(0.0, 0.05)
    row_num[2] = -1.0 + rng.normal(0.0, 0.05)
    col_den = np.concatenate(([1.0], rng.normal(0.0, 1e-4, 19)))
    row_den = np.concatenate(([1.0], rng.normal(0.0, 1e-4, 19)))
    rpc = {
        'rowOff': height / 2.0, 'rowScale': height / 2.0,
        'colOff': width / 2.0, 'colScale': width / 2.0,
        'latOff': float(rng.uniform(20.0, 50.0)), 'latScale': 0.05,
        'lonOff': float(rng.uniform(-120.0, 120.0)), 'lonScale': 0.05,
        'altOff': float(rng.uniform(0.0, 500.0)), 'altScale': 500.0,
        'rowNum': [float(v) for v in row_num], 'rowDen': [float(v) for v in row_den],
        'colNum': [float(v) for v in col_num], 'colDen': [float(v) for v in col_den],
    }
    return {'rpc': rpc, 'width': width, 'height': height}


def grid_points(x_points: np.ndarray, y_points: np.ndarray, z_points: np.ndarray):
    """3-D sample grid in the layout of ``lib/gen_grid.py:38-56``.

    Points are z-major; inside one z slab the (x, y) pairs follow an ``ij`` meshgrid
    flattened row-major.  Returns three (N, 1) float64 columns.
    """
    nx, ny, nz = x_points.size, y_points.size, z_points.size
    slab_x = np.repeat(np.asarray(x_points, dtype=np.float64), ny)
    slab_y = np.tile(np.asarray(y_points, dtype=np.float64), nx)
    xx = np.tile(slab_x, nz).reshape(-1, 1)
    yy = np.tile(slab_y, nz).reshape(-1, 1)
    zz = np.repeat(np.asarray(z_points, dtype=np.float64), nx * ny).reshape(-1, 1)
    return xx, yy, zz


@dataclass
class SampleGrid:
    """A lat/lon/alt sample grid and its ENU coordinates, each (N, 1) float64."""
    lat: np.ndarray
    lon: np.ndarray
    alt: np.ndarray
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    origin: tuple

    @property
    def n(self) -> int:
        return self.lat.shape[0]


def rpc_sample_grid(meta: dict, n_xy: int, n_z: int) -> SampleGrid:
    """Grid over the camera's normalised cube [-1, 1]^3 converted to degrees and metres.

    Latitude runs north to south and longitude west to east, as the northing/easting
    linspaces of ``camera_approx.py:66-70`` do.  ENU is taken about the grid's centre
    latitude/longitude at its lowest altitude (``coordinate_system.py:45-47``).
    """
    r = meta['rpc']
    lat_pts = r['latOff'] + r['latScale'] * np.linspace(1.0, -1.0, n_xy)
    lon_pts = r['lonOff'] + r['lonScale'] * np.linspace(-1.0, 1.0, n_xy)
    alt_pts = r['altOff'] + r['altScale'] * np.linspace(-1.0, 1.0, n_z)
    lat, lon, alt = grid_points(lat_pts, lon_pts, alt_pts)
    lat0 = (lat_pts.min() + lat_pts.max()) / 2.0
    lon0 = (lon_pts.min() + lon_pts.max()) / 2.0
    alt0 = float(alt_pts.min())
    x, y, z = geodetic_to_enu(lat, lon, alt, lat0, lon0, alt0)
    return SampleGrid(lat, lon, alt, x, y, z, (lat0, lon0, alt0))


def normalized_cube(seed: int, n: int):
    """N points uniform over the normalised cube [-1, 1]^3 as float32 (x=lat, y=lon, z=alt)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, size=(3, n)).astype(np.float32)


# --------------------------------------------------------------------------------------
# Height-map scenes and per-view point clouds
# --------------------------------------------------------------------------------------
@dataclass
class DsmGrid:
    """DSM grid spec, the arguments of ``proj_to_grid`` (``lib/proj_to_grid.py:41``)."""
    xoff: float      # upper-left easting
    yoff: float      # upper-left northing
    xres: float
    yres: float
    xsize: int
    ysize: int


@dataclass
class Scene:
    """A box-city scene: axis-aligned boxes in UTM over a flat ground at 0 m."""
    grid: DsmGrid
    boxes: np.ndarray   # (B, 5) float64: e0, e1, n0, n1, height (box covers e0<=E<e1, n0<=N<n1)
    noise: float


def make_scene(seed: int, grid: DsmGrid, n_boxes: int, h_lo: float, h_hi: float,
               noise: float = 0.3) -> Scene:
    rng = np.random.default_rng(seed)
    w = grid.xsize * grid.xres
    h = grid.ysize * grid.yres
    side_e = rng.uniform(4.0, 40.0, n_boxes)
    side_n = rng.uniform(4.0, 40.0, n_boxes)
    ce = grid.xoff + rng.uniform(0.0, w, n_boxes)
    cn = grid.yoff - rng.uniform(0.0, h, n_boxes)
    hh = rng.uniform(h_lo, h_hi, n_boxes)
    boxes = np.stack([ce - side_e / 2, ce + side_e / 2, cn - side_n / 2, cn + side_n / 2, hh], axis=1)
    return Scene(grid, boxes, noise)


@dataclass
class ViewSpec:
    """Pixel -> UTM affine map and corruption of one synthetic height map."""
    height: int
    width: int
    gsd: float          # metres per pixel
    theta: float        # rotation (radians)
    shift_e: float      # per-view jitter of the UL corner (metres)
    shift_n: float
    nan_frac: float
    seed: int


def make_views(seed: int, scene: Scene, n_views: int, height: int, width: int,
               nan_lo: float, nan_hi: float, jitter: float) -> list:
    """Per-view specs whose footprint covers the scene's DSM grid (6% margin, so the
    small rotations and shifts leave no uncovered corners)."""
    rng = np.random.default_rng(seed)
    g = scene.grid
    gsd = 1.06 * max(g.xsize * g.xres / width, g.ysize * g.yres / height)
    views = []
    for v in range(n_views):
        views.append(ViewSpec(height, width, gsd,
                              theta=float(rng.uniform(-0.03, 0.03)),
                              shift_e=float(rng.uniform(-jitter, jitter)),
                              shift_n=float(rng.uniform(-jitter, jitter)),
                              nan_frac=float(rng.uniform(nan_lo, nan_hi)),
                              seed=int(seed * 1000 + v)))
    return views


_SCENE_CACHE = {}


def scene_raster_torch(scene: Scene, device='cpu'):
    """The scene's height field on a raster 4x finer than the DSM grid (plus a 10% margin),
    boxes painted once; returns (raster, e0, n0, step) with raster[i, j] the height at
    easting e0 + (j + 0.5) * step, northing n0 - (i + 0.5) * step."""
    import torch
    key = (id(scene), str(device))
    hit = _SCENE_CACHE.get(key)
    if hit is not None and hit[0] is scene:
        return hit[1]
    g = scene.grid
    step = min(g.xres, g.yres) / 4.0
    w = g.xsize * g.xres
    h = g.ysize * g.yres
    e0 = g.xoff - 0.1 * w
    n0 = g.yoff + 0.1 * h
    nx = int(math.ceil(1.2 * w / step))
    ny = int(math.ceil(1.2 * h / step))
    ras = torch.zeros((ny, nx), dtype=torch.float32, device=device)
    for b in range(scene.boxes.shape[0]):
        be0, be1, bn0, bn1, hb = scene.boxes[b].tolist()
        j0 = max(int(math.ceil((be0 - e0) / step - 0.5)), 0)
        j1 = min(int(math.ceil((be1 - e0) / step - 0.5)), nx)
        i0 = max(int(math.ceil((n0 - bn1) / step - 0.5)), 0)
        i1 = min(int(math.ceil((n0 - bn0) / step - 0.5)), ny)
        if j0 < j1 and i0 < i1:
            ras[i0:i1, j0:j1].clamp_(min=float(hb))
    out = (ras, e0, n0, step)
    _SCENE_CACHE[key] = (scene, out)
    return out


def view_points_torch(scene: Scene, view: ViewSpec, device='cpu'):
    """(H*W, 3) float64 torch tensor of (easting, northing, height) for one view.

    Each pixel is mapped to UTM by the view's affine map; its height is the scene height
    there (tallest box, 0 m ground elsewhere) plus N(0, noise), and NaN with probability
    ``nan_frac``.  Rows follow the pixel raster, like the depth-map point lists of
    ``aggregate_2p5d_util.py:75-98``.
    """
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(view.seed)
    H, W = view.height, view.width
    g = scene.grid
    f64 = torch.float64
    ras, e0, n0, step = scene_raster_torch(scene, device)
    jj = torch.arange(W, device=device, dtype=f64) + 0.5
    ii = torch.arange(H, device=device, dtype=f64) + 0.5
    c, s = math.cos(view.theta), math.sin(view.theta)
    # rotate about the image centre so every view covers the grid
    dj = (jj - W / 2.0)[None, :]
    di = (ii - H / 2.0)[:, None]
    ce = g.xoff + g.xsize * g.xres / 2.0 + view.shift_e
    cn = g.yoff - g.ysize * g.yres / 2.0 + view.shift_n
    east = ce + view.gsd * (c * dj - s * di)
    north = cn - view.gsd * (s * dj + c * di)
    ci = ((east - e0) / step).floor().long()
    ri = ((n0 - north) / step).floor().long()
    inside = (ci >= 0) & (ci < ras.shape[1]) & (ri >= 0) & (ri < ras.shape[0])
    height = ras[ri.clamp(0, ras.shape[0] - 1), ci.clamp(0, ras.shape[1] - 1)]
    height = torch.where(inside, height, torch.zeros_like(height))
    noise = torch.randn((H, W), generator=gen, device=device, dtype=torch.float32) * scene.noise
    height = height + noise
    nan_mask = torch.rand((H, W), generator=gen, device=device) < view.nan_frac
    height = torch.where(nan_mask, torch.full_like(height, float('nan')), height)
    pts = torch.stack([east.reshape(-1), north.reshape(-1), height.reshape(-1).to(f64)], dim=1)
    return pts.contiguous()


def view_points(scene: Scene, view: ViewSpec) -> np.ndarray:
    """numpy (H*W, 3) float64 point list of one view (CPU generation)."""
    return view_points_torch(scene, view, 'cpu').numpy()


# --------------------------------------------------------------------------------------
# Named workloads
# --------------------------------------------------------------------------------------
def small_raster_case(seed: int = BASE_SEED):
    """One 1024x1024 FP32 height map (40 boxes 5-60 m, N(0,0.3) noise, 15% NaN) rasterised
    into a 0.5 m DSM anchored at the Explorer AOI's UL corner."""
    grid = DsmGrid(EXPLORER_UL_EASTING, EXPLORER_UL_NORTHING, 0.5, 0.5, 1025, 1025)
    scene = make_scene(seed + 1, grid, 40, 5.0, 60.0)
    view = ViewSpec(1024, 1024, 0.5, theta=0.02, shift_e=0.0, shift_n=0.0, nan_frac=0.15,
                    seed=seed + 2)
    return scene, view


def aoi50_raster_case(seed: int = BASE_SEED, n_views: int = 50, image: int = 4096,
                      cells: int = 2000, res: float = 0.3):
    """50 views of 4096x4096 FP32 height maps of one scene (300 boxes 3-80 m, 0.5 m view
    jitter, 10-20% NaN) rasterised to a 2000x2000 grid at 0.3 m."""
    grid = DsmGrid(EXPLORER_UL_EASTING, EXPLORER_UL_NORTHING, res, res, cells, cells)
    scene = make_scene(seed + 11, grid, 300, 3.0, 80.0)
    views = make_views(seed + 12, scene, n_views, image, image, 0.10, 0.20, 0.5)
    return scene, views


# --------------------------------------------------------------------------------------
# Many AOIs with per-view height maps (the batched and served forms)
# --------------------------------------------------------------------------------------
MAP_FRAC_BITS = 28


def map_affine(ce: float, cn: float, gsd: float, theta: float) -> dict:
    """Fixed-point (2^-28 m) pixel -> UTM map of a W x H view: pixel centres on a grid of
    spacing ``gsd`` rotated by ``theta`` about the image centre (ce, cn), rows running
    south.  Pixel (i, j) lands at e0 + ej(2j+1-W) + ei(2i+1-H) (and likewise north)."""
    s = float(1 << MAP_FRAC_BITS)
    c, sn = math.cos(theta), math.sin(theta)
    return {'e0': int(round(ce * s)), 'n0': int(round(cn * s)), 'ej': int(round(gsd * c / 2 * s)),
            'ei': int(round(-gsd * sn / 2 * s)), 'nj': int(round(-gsd * sn / 2 * s)),
            'ni': int(round(-gsd * c / 2 * s))}


@dataclass
class AoiSpec:
    """One AOI of the batched workload: its DSM grid, views and image size."""
    index: int
    xoff: float
    yoff: float
    res: float
    xsize: int
    ysize: int
    n_views: int
    image: int
    seed: int

    def grid(self) -> DsmGrid:
        return DsmGrid(self.xoff, self.yoff, self.res, self.res, self.xsize, self.ysize)

    @property
    def cells(self) -> int:
        return self.xsize * self.ysize


def make_aoi_set(n_aois: int = 200, seed: int = BASE_SEED, area_km2=(0.2, 4.0), views=(8, 60),
                 image=(1024, 8192), res=(0.3, 1.0)) -> list:
    """AOIs with footprint U(area_km2) km^2 (aspect U(0.75, 1.33)), grid resolution U(res)
    m, U{views} views and square images of U{image} px.  Origins lie in UTM-like ranges
    (easting 270-515 km, northing 4.2-8.38 Mm) that keep each grid inside one binade of
    its origin."""
    rng = np.random.default_rng(seed + 300)
    specs = []
    for a in range(n_aois):
        area = rng.uniform(*area_km2) * 1e6
        aspect = rng.uniform(0.75, 1.33)
        w_m = math.sqrt(area * aspect)
        h_m = area / w_m
        r = float(rng.uniform(*res))
        xsize, ysize = int(w_m / r) + 1, int(h_m / r) + 1
        xoff = float(rng.uniform(270000.0, 515000.0 - xsize * r))
        yoff = float(rng.uniform(4200000.0 + ysize * r, 8380000.0))
        n_views = int(rng.integers(views[0], views[1] + 1))
        img = int(rng.integers(image[0], image[1] + 1))
        specs.append(AoiSpec(a, xoff, yoff, r, xsize, ysize, n_views, img, seed + 7919 * (a + 1)))
    return specs


def aoi_view_affines(spec: AoiSpec, width: int = None, height: int = None, jitter: float = 0.5) -> list:
    """Per-view fixed-point affine maps whose footprint covers the AOI grid (6% margin),
    with a small rotation and a corner jitter, as ``make_views`` does for one AOI."""
    rng = np.random.default_rng(spec.seed)
    W = width or spec.image
    H = height or spec.image
    gsd = 1.06 * max(spec.xsize * spec.res / W, spec.ysize * spec.res / H)
    ce0 = spec.xoff + spec.xsize * spec.res / 2.0
    cn0 = spec.yoff - spec.ysize * spec.res / 2.0
    out = []
    for _ in range(spec.n_views):
        theta = float(rng.uniform(-0.03, 0.03))
        ce = ce0 + float(rng.uniform(-jitter, jitter))
        cn = cn0 + float(rng.uniform(-jitter, jitter))
        out.append(map_affine(ce, cn, gsd, theta))
    return out


def height_map_pool(n_maps: int, size: int, seed: int = BASE_SEED, device='cpu', n_boxes: int = 300,
                    h_lo: float = 3.0, h_hi: float = 80.0, noise: float = 0.3, nan_lo: float = 0.10,
                    nan_hi: float = 0.20):
    """(n_maps, size, size) float32 height maps as in the single-AOI workload: ground 0 m,
    ``n_boxes`` boxes (sides 1.5-15% of the map) of height U(h_lo, h_hi), N(0, noise)
    noise, and NaN on a U(nan_lo, nan_hi) fraction of the pixels."""
    import torch
    rng = np.random.default_rng(seed + 500)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed + 501)
    pool = torch.zeros((n_maps, size, size), dtype=torch.float32, device=device)
    for m in range(n_maps):
        lo, hi = max(2, int(0.015 * size)), max(3, int(0.15 * size))
        sides = rng.integers(lo, hi, size=(n_boxes, 2))
        corners = rng.integers(0, size, size=(n_boxes, 2))
        heights = rng.uniform(h_lo, h_hi, n_boxes)
        for b in range(n_boxes):
            i0, j0 = int(corners[b, 0]), int(corners[b, 1])
            pool[m, i0:i0 + int(sides[b, 0]), j0:j0 + int(sides[b, 1])].clamp_(min=float(heights[b]))
        pool[m] += torch.randn((size, size), generator=gen, device=device) * noise
        frac = float(rng.uniform(nan_lo, nan_hi))
        pool[m].masked_fill_(torch.rand((size, size), generator=gen, device=device) < frac, float('nan'))
    return pool


def small_aoi_case(seed: int = BASE_SEED):
    """Three small AOIs (2-4 views each) for parity tests: per-view (H, W) float32 maps with
    NaN, signed zeros and odd widths, and their grids and affine maps."""
    rng = np.random.default_rng(seed + 900)
    specs = [AoiSpec(0, 354052.25, 6182702.5, 0.5, 41, 33, 3, 0, seed + 1),
             AoiSpec(1, 300001.0, 4300123.75, 0.3, 64, 64, 3, 0, seed + 2),
             AoiSpec(2, 512000.5, 8200000.0, 1.0, 27, 50, 4, 0, seed + 3)]
    maps, affines = [], []
    for s in specs:
        ms, afs = [], []
        sizes = [(int(rng.integers(30, 70)), int(rng.integers(30, 70))) for _ in range(s.n_views)]
        for v in range(s.n_views):
            H, W = sizes[v]
            m = (rng.normal(0.0, 0.3, (H, W)) + rng.choice([0.0, 10.0, 25.0], (H, W), p=[0.6, 0.3, 0.1]))
            m = m.astype(np.float32)
            m[rng.random((H, W)) < 0.15] = np.nan
            zeros = rng.random((H, W)) < 0.03
            m[zeros] = np.where(rng.random(zeros.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
            ms.append(m)
            sub = AoiSpec(s.index, s.xoff, s.yoff, s.res, s.xsize, s.ysize, 1, 0, s.seed + 31 * v)
            afs.append(aoi_view_affines(sub, width=W, height=H)[0])
        maps.append(ms)
        affines.append(afs)
    return specs, maps, affines


def rpc_sample_grid_torch(meta: dict, n_xy: int, n_z: int, device='cpu') -> dict:
    """``rpc_sample_grid`` on a torch device: flat FP64 tensors lat, lon, alt, x, y, z (the
    same grid order and the same ENU formulas, in torch operations)."""
    import torch
    f64 = torch.float64
    r = meta['rpc']
    lat_pts = r['latOff'] + r['latScale'] * torch.linspace(1.0, -1.0, n_xy, dtype=f64, device=device)
    lon_pts = r['lonOff'] + r['lonScale'] * torch.linspace(-1.0, 1.0, n_xy, dtype=f64, device=device)
    alt_pts = r['altOff'] + r['altScale'] * torch.linspace(-1.0, 1.0, n_z, dtype=f64, device=device)
    lat = lat_pts.repeat_interleave(n_xy).repeat(n_z)
    lon = lon_pts.repeat(n_xy).repeat(n_z)
    alt = alt_pts.repeat_interleave(n_xy * n_xy)
    lat0 = float((lat_pts.min() + lat_pts.max()) / 2.0)
    lon0 = float((lon_pts.min() + lon_pts.max()) / 2.0)
    alt0 = float(alt_pts.min())

    def ecef(la, lo, al):
        phi, lam = torch.deg2rad(torch.as_tensor(la, dtype=f64, device=device)), \
            torch.deg2rad(torch.as_tensor(lo, dtype=f64, device=device))
        sphi = torch.sin(phi)
        n = 6378137.0 / torch.sqrt(1.0 - _E2 * sphi * sphi)
        return ((n + al) * torch.cos(phi) * torch.cos(lam), (n + al) * torch.cos(phi) * torch.sin(lam),
                (n * (1.0 - _E2) + al) * sphi)

    x, y, z = ecef(lat, lon, alt)
    x0, y0, z0 = ecef(lat0, lon0, alt0)
    dx, dy, dz = x - x0, y - y0, z - z0
    phi0, lam0 = math.radians(lat0), math.radians(lon0)
    sp, cp, sl, cl = math.sin(phi0), math.cos(phi0), math.sin(lam0), math.cos(lam0)
    east = -sl * dx + cl * dy
    t = cl * dx + sl * dy
    north = -sp * t + cp * dz
    up = cp * t + sp * dz
    return {'lat': lat, 'lon': lon, 'alt': alt, 'x': east, 'y': north, 'z': up}


_E2 = (1.0 / 298.257223563) * (2.0 - 1.0 / 298.257223563)


def aoi_rpc_metas(spec: AoiSpec) -> list:
    """Per-view RPC cameras of one AOI: independent seeded coefficients (as
    ``make_rpc_meta``) around one shared normalisation (the AOI's lat/lon/alt offsets), so
    every view sees the AOI's sample grid."""
    base = make_rpc_meta(spec.seed, spec.image, spec.image)
    out = []
    for v in range(spec.n_views):
        m = make_rpc_meta(spec.seed + 1 + v, spec.image, spec.image)
        for k in ('latOff', 'latScale', 'lonOff', 'lonScale', 'altOff', 'altScale'):
            m['rpc'][k] = base['rpc'][k]
        out.append(m)
    return out


def _loguniform(rng, lo, hi):
    return float(math.exp(rng.uniform(math.log(lo), math.log(hi))))


def make_aoi_catalog(n_aois: int = 400, seed: int = BASE_SEED, area_km2=(0.2, 4.0), views=(8, 60),
                     image=(1024, 8192), res=(0.3, 1.0)) -> list:
    """AOIs of the serving workload: the ranges of ``make_aoi_set`` drawn log-uniformly
    (footprint, resolution, view count and image size)."""
    rng = np.random.default_rng(seed + 700)
    specs = []
    for a in range(n_aois):
        area = _loguniform(rng, *area_km2) * 1e6
        aspect = rng.uniform(0.75, 1.33)
        w_m = math.sqrt(area * aspect)
        h_m = area / w_m
        r = _loguniform(rng, *res)
        xsize, ysize = int(w_m / r) + 1, int(h_m / r) + 1
        xoff = float(rng.uniform(270000.0, 515000.0 - xsize * r))
        yoff = float(rng.uniform(4200000.0 + ysize * r, 8380000.0))
        n_views = int(round(_loguniform(rng, views[0], views[1])))
        img = int(round(_loguniform(rng, image[0], image[1])))
        specs.append(AoiSpec(a, xoff, yoff, r, xsize, ysize, n_views, img, seed + 104729 * (a + 1)))
    return specs


# --------------------------------------------------------------------------------------
# Depth maps of satellite-like perspective views (the depth map -> UTM points chain)
# --------------------------------------------------------------------------------------
@dataclass
class DepthCase:
    """An AOI (the reference's aoi.json fields), a box-city scene in ENU metres about the
    AOI origin, and per-view 4x4 inverse projection matrices as COLMAP's inv_proj_mats.txt
    holds them (``aggregate_2p5d_util.py:55-61``)."""
    aoi: dict
    scene: Scene
    inv_proj: np.ndarray     # (V, 4, 4) float64
    height: int
    width: int
    nan_frac: list
    seeds: list


def make_depth_case(seed: int, n_views: int, height: int, width: int, utm_fn, aoi_m: float = 600.0,
                    lat0: float = 39.77, lon0: float = -84.05, n_boxes: int = 300) -> DepthCase:
    """Views of a square AOI of side ``aoi_m`` from cameras 550-650 km away, 5-30 degrees off
    nadir: P = K [R | -R C] in ENU, extended with a [0 0 0 1] row and inverted (so the
    "depth" of a pixel is the reciprocal of its projective scale).  ``utm_fn(lat, lon, zone,
    south) -> (east, north)`` places the AOI's upper-left UTM corner (ul_easting,
    ul_northing) from its centre."""
    from .coordinate_system import utm_zone
    rng = np.random.default_rng(seed)
    dlat = aoi_m / 2.0 / 111132.954
    dlon = aoi_m / 2.0 / (111319.49 * math.cos(math.radians(lat0)))
    zone = utm_zone(lat0, lon0)
    south = lat0 < 0
    ec, nc = utm_fn(lat0, lon0, zone, south)
    aoi = {'lat_min': lat0 - dlat, 'lat_max': lat0 + dlat, 'lon_min': lon0 - dlon, 'lon_max': lon0 + dlon,
           'alt_min': -30.0, 'alt_max': 120.0, 'width': aoi_m, 'height': aoi_m,
           'ul_easting': float(np.floor(float(ec) - aoi_m / 2.0)),
           'ul_northing': float(np.floor(float(nc) + aoi_m / 2.0)),
           'zone_number': zone, 'hemisphere': 'S' if south else 'N'}
    grid = DsmGrid(-aoi_m / 2.0, aoi_m / 2.0, 0.5, 0.5, int(aoi_m / 0.5), int(aoi_m / 0.5))
    scene = make_scene(seed + 1, grid, n_boxes, 3.0, 80.0, noise=0.2)
    mats, fracs, seeds = [], [], []
    for v in range(n_views):
        off = math.radians(rng.uniform(5.0, 30.0))
        az = rng.uniform(0.0, 2.0 * math.pi)
        dist = rng.uniform(550e3, 650e3)
        target = np.array([rng.uniform(-20, 20), rng.uniform(-20, 20), 30.0])
        C = target + dist * np.array([math.sin(off) * math.sin(az), math.sin(off) * math.cos(az), math.cos(off)])
        z = (target - C) / np.linalg.norm(target - C)
        x = np.cross(z, [0.0, 1.0, 0.0])
        x /= np.linalg.norm(x)
        y = np.cross(z, x)
        roll = rng.uniform(-0.1, 0.1)
        x, y = math.cos(roll) * x + math.sin(roll) * y, -math.sin(roll) * x + math.cos(roll) * y
        R = np.stack([x, y, z])
        f = width * dist / (1.15 * aoi_m)
        K = np.array([[f, rng.normal(0.0, 1.0), width / 2.0], [0.0, f * rng.uniform(0.999, 1.001), height / 2.0],
                      [0.0, 0.0, 1.0]])
        P4 = np.eye(4)
        P4[:3, :3] = K @ R
        P4[:3, 3] = -K @ R @ C
        mats.append(np.linalg.inv(P4))
        fracs.append(float(rng.uniform(0.10, 0.20)))
        seeds.append(int(seed * 1000 + v))
    return DepthCase(aoi, scene, np.stack(mats), height, width, fracs, seeds)


def depth_map_torch(case: DepthCase, v: int, device='cpu'):
    """(H, W) float32 depth map of view v: each pixel's depth puts its point on the scene
    surface (the ray meets up = 0, the scene height there plus N(0, noise) is looked up, and
    the depth solving up = height is taken), rounded to float32; ``nan_frac`` of the pixels
    are invalid (COLMAP's -1e20, a few exact zeros)."""
    import torch
    f64 = torch.float64
    H, W = case.height, case.width
    M = torch.tensor(case.inv_proj[v], dtype=f64, device=device)
    gen = torch.Generator(device=device)
    gen.manual_seed(case.seeds[v])
    cc = torch.arange(W, device=device, dtype=f64)[None, :]
    rr = torch.arange(H, device=device, dtype=f64)[:, None]
    a = [M[i, 0] * cc + M[i, 1] * rr + M[i, 2] for i in range(4)]
    b = [M[i, 3] for i in range(4)]
    d0 = -a[2] / b[2]                                        # up = 0 (w = a3 + b3 d)
    w0 = a[3] + b[3] * d0
    e = (a[0] + b[0] * d0) / w0
    n = (a[1] + b[1] * d0) / w0
    ras, e0, n0, step = scene_raster_torch(case.scene, device)
    ci = ((e - e0) / step).floor().long()
    ri = ((n0 - n) / step).floor().long()
    inside = (ci >= 0) & (ci < ras.shape[1]) & (ri >= 0) & (ri < ras.shape[0])
    h = ras[ri.clamp(0, ras.shape[0] - 1), ci.clamp(0, ras.shape[1] - 1)].to(f64)
    h = torch.where(inside, h, torch.zeros_like(h))
    h = h + torch.randn((H, W), generator=gen, device=device, dtype=f64) * case.scene.noise
    d = ((h * a[3] - a[2]) / (b[2] - h * b[3])).to(torch.float32)
    u = torch.rand((H, W), generator=gen, device=device)
    d = torch.where(u < case.nan_frac[v], torch.full_like(d, -1e20), d)
    d = torch.where(u < 0.01 * case.nan_frac[v], torch.zeros_like(d), d)
    return d.contiguous()
