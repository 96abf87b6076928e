"""On-disk formats (CPU): PLY bytes against the reference's np2ply outputs, and the GeoTIFF
writer/reader round trip (parity with GDAL unpinned: GDAL is not installed)."""
import os

import numpy as np

from conftest import same_bits

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def test_ply_binary_bytes_match_reference(tmp_path):
    from vissatsatellitestereo_gb300 import io_formats as io
    z = np.load(os.path.join(GOLDEN, 'ply_inputs.npz'))
    v, c = z['vertex'], z['color']
    cases = {'ply_f32.ply': {}, 'ply_f32_color.ply': dict(color=c, comments=['VisSat point cloud', 'utm 17N']),
             'ply_f64.ply': dict(use_double=True)}
    for name, kw in cases.items():
        out = tmp_path / name
        io.np2ply(v, str(out), **kw)
        assert out.read_bytes() == open(os.path.join(GOLDEN, name), 'rb').read(), name
        vv, cc, com = io.read_ply(str(out))
        assert np.array_equal(vv, v.astype(np.float64 if kw.get('use_double') else np.float32))
        assert (cc is None) == ('color' not in kw)


def test_ply_text_mode(tmp_path):
    from vissatsatellitestereo_gb300 import io_formats as io
    v = np.array([[1.23456, -2.5, 3.0], [4.0, 5.5, -6.25]])
    c = np.array([[1, 2, 3], [250, 251, 252]], dtype=np.uint8)
    io.np2ply(v, str(tmp_path / 't.ply'), color=c, text=True)
    txt = (tmp_path / 't.ply').read_text().splitlines()
    assert txt[1] == 'format ascii 1.0' and txt[-2] == '1.2346 -2.5000 3.0000 1 2 3'
    vv, cc, _ = io.read_ply(str(tmp_path / 't.ply'))
    assert np.allclose(vv, np.round(v, 4)) and np.array_equal(cc, c)


def test_geotiff_round_trip(tmp_path):
    from vissatsatellitestereo_gb300 import io_formats as io
    rng = np.random.default_rng(2)
    img = rng.normal(30, 20, (301, 259)).astype(np.float32)
    img[rng.random(img.shape) < 0.2] = np.nan
    f = str(tmp_path / 'dsm.tif')
    io.write_dsm_tif(img, f, (354052.25, 6182702.5, 0.5, 0.5), (17, 'N'), nodata_val=-10000)
    back, meta = io.read_dsm_tif(f)
    assert same_bits(back, img)
    assert meta['img_width'] == 259 and meta['img_height'] == 301 and meta['nodata'] == -10000.0
    assert (meta['zone_number'], meta['hemisphere']) == (17, 'N')
    assert meta['geo'] == (354052.25, 0.5, 0.0, 6182702.5, 0.0, -0.5)
    assert meta['lr_easting'] == 354052.25 + 258 * 0.5 and meta['area_height'] == 300 * 0.5
    raw = open(f, 'rb').read()
    assert raw[:4] == b'II*\0' and b'AREA_OR_POINT' in raw and b'UTM zone 17N' in raw
    io.write_dsm_tif(img, f, (500000.0, 4000000.0, 1.0, 1.0), (33, 'S'))
    back, meta = io.read_dsm_tif(f)
    assert same_bits(back, img) and (meta['zone_number'], meta['hemisphere']) == (33, 'S')
