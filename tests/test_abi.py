"""The C ABI: the library builds/loads and exports every symbol the header declares (CPU)."""
import os
import re

import pytest

from conftest import ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, 'include', 'vissat_gb300.h')).read()
    txt = re.sub(r'/\*.*?\*/', '', txt, flags=re.S)
    return sorted(set(re.findall(r'\b(vs_\w+)\s*\(', txt)))


def test_header_declares_the_boundary():
    syms = header_symbols()
    for name in ('vs_rpc_project', 'vs_dlt_fit', 'vs_perspective_error', 'vs_camera_approx_perspective',
                 'vs_proj_to_grid', 'vs_dsm_from_points', 'vs_median_blur3x3_f32', 'vs_fuse_dsms'):
        assert name in syms


def test_library_exports_every_declared_symbol():
    from vissatsatellitestereo_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from vissatsatellitestereo_gb300.build import build
        build()
    lib = _lib.lib()
    for name in header_symbols():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f'{name} has no ctypes signature'
    assert lib.vs_version().decode().startswith('vissat-gb300')


def header_declarations():
    txt = open(os.path.join(ROOT, 'include', 'vissat_gb300.h')).read()
    txt = re.sub(r'/\*.*?\*/', '', txt, flags=re.S)
    txt = re.sub(r'//[^\n]*', '', txt)
    out = {}
    for name, params in re.findall(r'\b(vs_\w+)\s*\(([^;{}]*?)\)\s*;', txt):
        out[name] = [p.strip() for p in params.split(',')] if params.strip() not in ('', 'void') else []
    return out


def test_ctypes_signatures_match_the_header():
    """Every declared entry point's ctypes binding has the header's parameter count, a
    pointer exactly where the header has one, and scalars of the header's width and kind."""
    import ctypes
    from vissatsatellitestereo_gb300 import _lib
    scalars = {'int': ctypes.c_int, 'int32_t': ctypes.c_int32, 'int64_t': ctypes.c_int64, 'unsigned': ctypes.c_uint,
               'size_t': ctypes.c_size_t, 'double': ctypes.c_double, 'float': ctypes.c_float}
    decls = header_declarations()
    assert len(decls) == len(header_symbols())
    for name, params in decls.items():
        _, args = _lib.SIGNATURES[name]
        assert len(params) == len(args), name
        for p, a in zip(params, args):
            is_ptr = a in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(a, type) and issubclass(a, ctypes._Pointer))
            assert ('*' in p) == is_ptr, (name, p, a)
            if '*' in p:
                continue
            t = re.sub(r'\s+\w+$', '', p.replace('const ', '')).strip()
            assert t in scalars, (name, p)
            assert ctypes.sizeof(scalars[t]) == ctypes.sizeof(a), (name, p, a)
            assert (t in ('double', 'float')) == (a in (ctypes.c_double, ctypes.c_float)), (name, p, a)


def test_workspace_queries_need_no_gpu():
    from vissatsatellitestereo_gb300 import _lib
    lib = _lib.lib()
    assert lib.vs_proj_to_grid_workspace_size(2000, 2000) >= 2000 * 2000 * 8
    assert lib.vs_fuse_dsms_workspace_size(10, 10) >= 400
    assert lib.vs_dlt_fit_workspace_size(0, 10) == 0
    assert lib.vs_camera_approx_workspace_size(50, 800000) > 50 * 800000 * 16
    assert lib.vs_rpc_project_cube_workspace_size(50) >= 25 * 32 * 64
    assert lib.vs_rpc_project_cube_workspace_size(0) == 0


def test_camera_array_layout():
    from vissatsatellitestereo_gb300 import _lib, synth
    meta = synth.make_rpc_meta(1, 4096, 2048)
    a = _lib.camera_array([meta, meta])
    assert a.shape == (2, _lib.CAMERA_DOUBLES)
    r = meta['rpc']
    assert a[0, 0] == r['rowOff'] and a[0, 3] == r['colScale'] and a[0, 10] == r['rowNum'][0]
    assert a[0, 50] == r['colNum'][0] and a[0, 70] == r['colDen'][0] and a[0, 90] == 4096 and a[0, 91] == 2048
    with pytest.raises(ValueError):
        bad = dict(meta, rpc=dict(r, rowNum=r['rowNum'][:19]))
        _lib.camera_array([bad])


def test_header_compiles_as_c_and_struct_layouts_match(tmp_path):
    """The boundary is plain C: the header compiles with a C compiler (-std=c99, all
    warnings as errors), and the structs the Python side mirrors have the same sizes."""
    import ctypes
    import shutil
    import subprocess
    from vissatsatellitestereo_gb300 import _lib
    from vissatsatellitestereo_gb300.batch import VsAoi, VsMapView
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    src = tmp_path / 'abi.c'
    src.write_text('#include "vissat_gb300.h"\n#include <stdio.h>\n'
                   'int main(void) {\n'
                   '  printf("%zu %zu %zu %zu\\n", sizeof(VsRpcCamera), sizeof(VsGeoFrame), sizeof(VsAoi),'
                   ' sizeof(VsMapView));\n  return 0;\n}\n')
    exe = tmp_path / 'abi'
    inc = os.path.join(ROOT, 'include')
    subprocess.run([cc, '-std=c99', '-Wall', '-Wextra', '-Werror', '-I', inc, str(src), '-o', str(exe)], check=True)
    sizes = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [_lib.CAMERA_DOUBLES * 8, ctypes.sizeof(_lib.VsGeoFrame), ctypes.sizeof(VsAoi),
                     ctypes.sizeof(VsMapView)]
