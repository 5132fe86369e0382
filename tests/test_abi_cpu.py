"""CPU checks of the C ABI library: it loads, exports every declared entry
point, reads OTF files like the reference, and fails cleanly (return 0, no
exit) on bad input without touching the GPU."""

import ctypes
import re
import struct
from pathlib import Path

import numpy as np
import pytest

from cudadecon_gb300 import synth

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions():
    text = (ROOT / "include" / "cudadecon.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    # prototypes: a name, a parameter list (default-argument macros nest one
    # level of parentheses) and a semicolon
    names = re.findall(r"([A-Za-z_]\w*)\s*\((?:[^;{}()]|\([^()]*\))*\)\s*;", text)
    return sorted(set(names))


def test_header_declares_reference_abi():
    names = _declared_functions()
    for ref in ["RL_interface_init", "RL_interface", "Deskew_interface", "Affine_interface",
                "Affine_interface_RA", "camcor_interface_init", "camcor_interface", "RL_cleanup",
                "cuda_reset", "get_output_nx", "get_output_ny", "get_output_nz", "get_version"]:
        assert ref in names


def test_library_exports_every_declared_symbol(cdx):
    L = cdx.lib()
    missing = [n for n in _declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_declared_function_count():
    names = _declared_functions()
    assert "RL_interface" in names and "cdx_batch_last_launch_count" in names
    assert len(names) >= 33


def test_batch_stack_layout_matches_header(cdx, tmp_path):
    """The ctypes mirror of struct cdx_batch_stack has the C layout."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f[0] for f in cdx.BatchStack._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include <stdbool.h>\n"
                   f'#include "{ROOT / "include" / "cudadecon.h"}"\n'
                   "int main(void) {\n"
                   '  printf("%zu\\n", sizeof(cdx_batch_stack));\n' +
                   "".join(f'  printf("%zu\\n", offsetof(cdx_batch_stack, {f}));\n' for f in fields) +
                   "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [ctypes.sizeof(cdx.BatchStack)] + [getattr(cdx.BatchStack, f).offset for f in fields]
    assert got == want


def test_version_string(cdx):
    assert cdx.lib().get_version().decode()


def test_fft_length_support(cdx):
    L = cdx.lib()
    for n in synth.smooth_sizes(2, 2048):
        assert L.cdx_fft_length_supported(n) == 1
    for n in (11, 13, 17, 22, 26, 1021):
        assert L.cdx_fft_length_supported(n) == 0


@pytest.mark.parametrize("fmt", ["tif", "cimg"])
def test_otf_file_roundtrip(cdx, tmp_path, fmt):
    tab = synth.gaussian_otf_table(129, 64, 1.5, 4.0)
    tab = tab * np.exp(1j * np.linspace(0, 1, tab.size).reshape(tab.shape)).astype(np.complex64)
    p = tmp_path / f"otf.{fmt}"
    synth.write_otf(p, tab)
    img = cdx.load_image(p)
    assert img.shape == (1, 129, 128)
    np.testing.assert_array_equal(img[0].view(np.complex64), tab.astype(np.complex64))


def test_multipage_uint16_tiff(cdx, tmp_path):
    a = np.random.default_rng(0).integers(0, 65535, size=(5, 7, 9)).astype(np.uint16)
    p = tmp_path / "s.tif"
    synth.write_tiff(p, a)
    img = cdx.load_image(p)
    np.testing.assert_array_equal(img, a.astype(np.float32))


def test_big_endian_float_tiff(cdx, tmp_path):
    a = np.random.default_rng(1).random((3, 4)).astype(">f4")
    h, w = a.shape
    data = a.tobytes()
    off = 8
    body = data
    ifd_off = off + len(body)
    hdr = b"MM\x00*" + struct.pack(">I", ifd_off)
    tags = [(256, 4, 1, w), (257, 4, 1, h), (258, 3, 1, 32), (259, 3, 1, 1), (273, 4, 1, off),
            (277, 3, 1, 1), (278, 4, 1, h), (279, 4, 1, len(data)), (339, 3, 1, 3)]
    ifd = struct.pack(">H", len(tags))
    for t, ty, c, v in tags:
        ifd += struct.pack(">HHIHH", t, ty, c, v, 0) if ty == 3 else struct.pack(">HHII", t, ty, c, v)
    ifd += struct.pack(">I", 0)
    p = tmp_path / "be.tif"
    p.write_bytes(hdr + body + ifd)
    img = cdx.load_image(p)
    np.testing.assert_array_equal(img[0], a.astype(np.float32))


def test_init_with_missing_otf_returns_zero(cdx, tmp_path):
    L = cdx.lib()
    rc = L.RL_interface_init(64, 64, 32, 0.1, 0.1, 0.1, 0.1, 0.0, 0.0, 0, False,
                             str(tmp_path / "nope.tif").encode())
    assert rc == 0
    assert b"OTF" in L.cdx_last_error()


def test_init_with_garbage_otf_returns_zero(cdx, tmp_path):
    p = tmp_path / "bad.tif"
    p.write_bytes(b"II*\x00\xff\xff\xff\x7f")
    L = cdx.lib()
    assert L.RL_interface_init(64, 64, 32, 0.1, 0.1, 0.1, 0.1, 0.0, 0.0, 0, False,
                               str(p).encode()) == 0


def test_rl_interface_before_init_returns_zero(cdx):
    L = cdx.lib()
    raw = np.zeros((4, 4, 4), np.uint16)
    out = np.zeros((4, 4, 4), np.float32)
    # no successful init in this process yet for a 4x4x4 grid: must fail cleanly
    L.RL_cleanup()
    rc = L.RL_interface(raw.ctypes.data_as(ctypes.POINTER(ctypes.c_ushort)), 4, 4, 4,
                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), None, 100.0, False,
                        False, 1, 0, 0, 0, 0.0, False, False)
    assert rc == 0
