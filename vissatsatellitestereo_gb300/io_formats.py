"""On-disk formats around the path: PLY point clouds, GeoTIFF DSMs, COLMAP dense arrays and
the inverse projection matrices.

* ``np2ply`` -- lib/ply_np_converter.py:38-67.  Binary output is byte-identical to the
  reference's (its vendored plyfile, little endian): the header lines, float32 (or
  float64) x, y, z and optional uchar red, green, blue per vertex.  The reference's text
  mode passes ``text_fmt`` to a plyfile that does not accept it and raises; here text
  mode writes plyfile's ASCII layout with the formats the reference asks for (%.4f, %i).
* ``write_dsm_tif`` / ``read_dsm_tif`` -- lib/dsm_util.py:122-159 and :49-99 without
  GDAL: a single-band float32 GeoTIFF (uncompressed strips) with the reference's
  geotransform (upper-left corner, east and north resolution), the GDAL nodata tag, the
  WGS 84 / UTM zone as the projected CRS (EPSG 326zz north, 327zz south) and
  AREA_OR_POINT=Area (PixelIsArea).  NaN is written as ``nodata_val`` when given; the
  reader turns values close to the nodata value back into NaN (np.isclose, as the
  reference) and returns the reference's meta dict fields.

* ``read_array`` / ``write_array`` -- colmap/read_dense.py:36-51: COLMAP's dense arrays
  (depth and normal maps), an ASCII "width&height&channels&" header and float32 values in
  column-major order; the reader returns the reference's (height, width[, channels]).
* ``read_inv_proj_mats`` / ``write_inv_proj_mats`` -- aggregate_2p5d_util.py:55-61: one
  line per image, its name and the 16 values of its 4x4 inverse projection matrix.

Device tensors are accepted and copied to the host once.
"""
import struct

import numpy as np


def _host(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


# ---- PLY -------------------------------------------------------------------------------
def np2ply(vertex, out_ply, color=None, comments=None, text=False, use_double=False):
    vertex = _host(vertex)
    vertex = vertex.astype(np.float64 if use_double else np.float32)
    vtype = 'f8' if use_double else 'f4'
    fields = [('x', '<' + vtype), ('y', '<' + vtype), ('z', '<' + vtype)]
    if color is not None:
        color = _host(color)
        fields += [('red', 'u1'), ('green', 'u1'), ('blue', 'u1')]
    n = vertex.shape[0]
    rec = np.empty(n, dtype=fields)
    rec['x'], rec['y'], rec['z'] = vertex[:, 0], vertex[:, 1], vertex[:, 2]
    if color is not None:
        rec['red'], rec['green'], rec['blue'] = (color[:, k].astype(np.uint8) for k in range(3))
    names = {'f4': 'float', 'f8': 'double'}
    lines = ['ply', 'format ' + ('ascii' if text else 'binary_little_endian') + ' 1.0']
    lines += ['comment ' + c for c in (comments or [])]
    lines.append(f'element vertex {n}')
    lines += [f'property {names[vtype]} {a}' for a in 'xyz']
    if color is not None:
        lines += [f'property uchar {c}' for c in ('red', 'green', 'blue')]
    lines.append('end_header')
    header = ('\n'.join(lines) + '\n').encode('ascii')
    with open(out_ply, 'wb') as f:
        f.write(header)
        if text:
            fmt = ['%.4f'] * 3 + (['%i'] * 3 if color is not None else [])
            for r in rec:
                f.write((' '.join(fm % v for fm, v in zip(fmt, r.tolist())) + '\n').encode('ascii'))
        else:
            f.write(rec.tobytes())


def read_ply(path):
    """(vertex (N, 3), color (N, 3) or None, comments) of a PLY file written by np2ply."""
    with open(path, 'rb') as f:
        data = f.read()
    end = data.index(b'end_header\n') + len(b'end_header\n')
    lines = data[:end].decode('ascii').split('\n')
    comments = [l[8:] for l in lines if l.startswith('comment ')]
    n = int(next(l for l in lines if l.startswith('element vertex')).split()[-1])
    props = [l.split()[1:] for l in lines if l.startswith('property ')]
    kinds = {'float': '<f4', 'double': '<f8', 'uchar': 'u1'}
    dtype = [(name, kinds[t]) for t, name in props]
    if 'ascii' in lines[1]:
        rows = [r.split() for r in data[end:].decode('ascii').strip().split('\n')][:n]
        rec = np.array([tuple(float(v) for v in r) for r in rows], dtype=[(a, '<f8') for _, a in props])
    else:
        rec = np.frombuffer(data[end:], dtype=dtype, count=n)
    vertex = np.stack([rec['x'], rec['y'], rec['z']], axis=1)
    color = np.stack([rec['red'], rec['green'], rec['blue']], axis=1) if 'red' in rec.dtype.names else None
    return vertex, color, comments


# ---- GeoTIFF ----------------------------------------------------------------------------
_TAGS = {'width': 256, 'height': 257, 'bits': 258, 'compression': 259, 'photometric': 262, 'strip_offsets': 273,
         'samples': 277, 'rows_per_strip': 278, 'strip_counts': 279, 'planar': 284, 'sample_format': 339,
         'pixel_scale': 33550, 'tiepoint': 33922, 'geokeys': 34735, 'geo_ascii': 34737, 'gdal_metadata': 42112,
         'gdal_nodata': 42113}
_SHORT, _LONG, _DOUBLE, _ASCII = 3, 4, 12, 2
_SIZE = {_SHORT: 2, _LONG: 4, _DOUBLE: 8, _ASCII: 1}


def _utm_epsg(zone_number, hemisphere):
    return (32600 if hemisphere == 'N' else 32700) + int(zone_number)


def write_dsm_tif(image, out_file, geo, utm_zone, nodata_val=None):
    """geo: (ul_e, ul_n, e_resolution, n_resolution); utm_zone: (zone number, 'N' or 'S')."""
    image = _host(image)
    assert image.ndim == 2
    ul_e, ul_n, e_res, n_res = (float(v) for v in geo)
    zone, hemi = utm_zone
    img = image.astype(np.float32)
    if nodata_val is not None:
        img = img.copy()
        img[np.isnan(img)] = nodata_val
    else:
        nodata_val = float('nan')
    h, w = img.shape
    rows_per_strip = max(1, min(h, (1 << 16) // max(1, w * 4)))
    strips = [img[r:r + rows_per_strip].astype('<f4').tobytes() for r in range(0, h, rows_per_strip)]
    epsg = _utm_epsg(zone, hemi)
    citation = f'WGS84 / UTM zone {zone}{hemi}|'
    # GeoKey directory: version 1.1.0; model type projected, raster type PixelIsArea,
    # projected CRS, citation (in the ASCII params)
    geokeys = [1, 1, 0, 4, 1024, 0, 1, 1, 1025, 0, 1, 1, 3072, 0, 1, epsg,
               3073, _TAGS['geo_ascii'], len(citation), 0]
    nodata_str = ('nan' if nodata_val != nodata_val else repr(float(nodata_val)).rstrip('0').rstrip('.')
                  if float(nodata_val) != int(nodata_val) else str(int(nodata_val))) + '\0'
    gdal_meta = '<GDALMetadata>\n  <Item name="AREA_OR_POINT">Area</Item>\n</GDALMetadata>\n\0'
    entries = [
        (_TAGS['width'], _LONG, [w]), (_TAGS['height'], _LONG, [h]), (_TAGS['bits'], _SHORT, [32]),
        (_TAGS['compression'], _SHORT, [1]), (_TAGS['photometric'], _SHORT, [1]),
        (_TAGS['strip_offsets'], _LONG, [0] * len(strips)), (_TAGS['samples'], _SHORT, [1]),
        (_TAGS['rows_per_strip'], _LONG, [rows_per_strip]),
        (_TAGS['strip_counts'], _LONG, [len(s) for s in strips]), (_TAGS['planar'], _SHORT, [1]),
        (_TAGS['sample_format'], _SHORT, [3]),
        (_TAGS['pixel_scale'], _DOUBLE, [e_res, n_res, 0.0]),
        (_TAGS['tiepoint'], _DOUBLE, [0.0, 0.0, 0.0, ul_e, ul_n, 0.0]),
        (_TAGS['geokeys'], _SHORT, geokeys), (_TAGS['geo_ascii'], _ASCII, citation + '\0'),
        (_TAGS['gdal_metadata'], _ASCII, gdal_meta), (_TAGS['gdal_nodata'], _ASCII, nodata_str),
    ]
    # layout: header (8) | IFD (entries sorted by tag) | out-of-line values | strips
    def raw_of(typ, vals):
        if typ == _ASCII:
            return vals.encode('ascii')
        return struct.pack('<' + {_SHORT: 'H', _LONG: 'I', _DOUBLE: 'd'}[typ] * len(vals), *vals)

    strip_idx = next(i for i, e in enumerate(entries) if e[0] == _TAGS['strip_offsets'])
    pos = 8 + 2 + 12 * len(entries) + 4
    where = {}
    for i, (tag, typ, vals) in enumerate(entries):
        size = len(raw_of(typ, vals))
        if size > 4:
            where[i] = pos
            pos += size + (size % 2)
    offsets, p = [], pos
    for st in strips:
        offsets.append(p)
        p += len(st)
    entries[strip_idx] = (_TAGS['strip_offsets'], _LONG, offsets)
    out = bytearray(b'II*\0' + struct.pack('<I', 8) + struct.pack('<H', len(entries)))
    blobs = bytearray()
    for i, (tag, typ, vals) in enumerate(entries):
        raw = raw_of(typ, vals)
        count = len(vals)
        if i in where:
            out += struct.pack('<HHII', tag, typ, count, where[i])
            blobs += raw + (b'\0' if len(raw) % 2 else b'')
        else:
            out += struct.pack('<HHI', tag, typ, count) + raw.ljust(4, b'\0')
    out += struct.pack('<I', 0) + blobs
    assert len(out) == pos
    for st in strips:
        out += st
    with open(out_file, 'wb') as f:
        f.write(bytes(out))


def read_dsm_tif(path):
    """(image float32 with nodata -> NaN, meta dict) of a GeoTIFF written by write_dsm_tif,
    with the fields of the reference's read_dsm_tif (lib/dsm_util.py:49-99)."""
    with open(path, 'rb') as f:
        data = f.read()
    assert data[:4] == b'II*\0'
    (ifd_off,) = struct.unpack_from('<I', data, 4)
    (n,) = struct.unpack_from('<H', data, ifd_off)
    tags = {}
    for k in range(n):
        tag, typ, count, val = struct.unpack_from('<HHII', data, ifd_off + 2 + 12 * k)
        size = _SIZE[typ] * count
        off = ifd_off + 2 + 12 * k + 8 if size <= 4 else val
        raw = data[off:off + size]
        if typ == _ASCII:
            tags[tag] = raw.decode('ascii').rstrip('\0')
        else:
            tags[tag] = list(struct.unpack('<' + {_SHORT: 'H', _LONG: 'I', _DOUBLE: 'd'}[typ] * count, raw))
    w, h = tags[_TAGS['width']][0], tags[_TAGS['height']][0]
    assert tags[_TAGS['bits']][0] == 32 and tags[_TAGS['sample_format']][0] == 3
    buf = b''.join(data[o:o + c] for o, c in zip(tags[_TAGS['strip_offsets']], tags[_TAGS['strip_counts']]))
    image = np.frombuffer(buf, dtype='<f4', count=w * h).reshape(h, w).astype(np.float32)
    nodata = float(tags[_TAGS['gdal_nodata']]) if _TAGS['gdal_nodata'] in tags else None
    if nodata is not None:
        image = image.copy()
        image[np.isclose(image, nodata)] = np.nan
    e_res, n_res = tags[_TAGS['pixel_scale']][:2]
    ul_e, ul_n = tags[_TAGS['tiepoint']][3:5]
    keys = tags[_TAGS['geokeys']]
    epsg = next(keys[4 + 4 * i + 3] for i in range(keys[3]) if keys[4 + 4 * i] == 3072)
    zone, hemi = epsg % 100, 'N' if epsg // 100 == 326 else 'S'
    meta = {'geo': (ul_e, e_res, 0.0, ul_n, 0.0, -n_res), 'img_width': w, 'img_height': h, 'nodata': nodata,
            'zone_number': zone, 'hemisphere': hemi, 'ul_easting': ul_e, 'ul_northing': ul_n,
            'east_resolution': e_res, 'north_resolution': abs(n_res)}
    meta['lr_easting'] = meta['ul_easting'] + (w - 1) * meta['east_resolution']
    meta['lr_northing'] = meta['ul_northing'] - (h - 1) * meta['north_resolution']
    meta['area_width'] = meta['lr_easting'] - meta['ul_easting']
    meta['area_height'] = meta['ul_northing'] - meta['lr_northing']
    with np.errstate(all='ignore'):
        meta['alt_min'] = float(np.nanmin(image)) if np.isfinite(image).any() else float('nan')
        meta['alt_max'] = float(np.nanmax(image)) if np.isfinite(image).any() else float('nan')
    return image, meta


# ---- COLMAP dense arrays and inverse projection matrices ---------------------------------
def read_array(path):
    """``colmap/read_dense.py:36-51``: an ASCII header "width&height&channels&" followed by
    float32 values in column-major (width, height, channels) order; returns (height, width)
    for one channel, (height, width, channels) otherwise, as the reference's squeeze does."""
    with open(path, 'rb') as f:
        raw = f.read()
    pos, fields = 0, []
    while len(fields) < 3:
        amp = raw.index(b'&', pos)
        fields.append(int(raw[pos:amp].decode().strip()))
        pos = amp + 1
    width, height, channels = fields
    arr = np.frombuffer(raw, dtype='<f4', offset=pos, count=width * height * channels)
    arr = arr.reshape((width, height, channels), order='F')
    return np.transpose(arr, (1, 0, 2)).squeeze()


def write_array(array, path):
    """Inverse of ``read_array`` (COLMAP's writer): (height, width[, channels]) float32."""
    a = _host(array).astype(np.float32)
    if a.ndim == 2:
        a = a[:, :, None]
    height, width, channels = a.shape
    with open(path, 'wb') as f:
        f.write(f'{width}&{height}&{channels}&'.encode())
        f.write(np.transpose(a, (1, 0, 2)).astype('<f4').tobytes(order='F'))


def read_inv_proj_mats(path):
    """``aggregate_2p5d_util.py:55-61``: one line per image, "name m00 m01 ... m33"
    (space-separated, row-major) -> {name: (4, 4) float64}."""
    mats = {}
    with open(path) as fp:
        for line in fp.readlines():
            tmp = line.split(' ')
            mats[tmp[0]] = np.array([float(tmp[i]) for i in range(1, 17)]).reshape((4, 4))
    return mats


def write_inv_proj_mats(mats, path):
    """Writes {name: (4, 4)} in the layout ``read_inv_proj_mats`` reads (repr of each float,
    so the values round-trip exactly)."""
    with open(path, 'w') as fp:
        for name, m in mats.items():
            vals = ' '.join(repr(float(x)) for x in np.asarray(m, dtype=np.float64).reshape(-1))
            fp.write(f'{name} {vals}\n')
