"""The C ABI: the built library loads and exports every entry point include/cfd3d.h declares;
host-side argument validation answers without a GPU."""
import ctypes as C
import os
import re

import pytest

from cfd3d_gb300 import abi, build, cases, native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "cfd3d.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cfd3d_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(build.build())
    names = declared()
    assert len(names) >= 16
    for n in names:
        assert hasattr(lib, n), n
    assert set(native.EXPORTS) == set(names)


def test_structs_match_header_layout(tmp_path):
    """The ctypes mirrors have the C compiler's sizes and field offsets for the header."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "l.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "%s"\n'
        'int main(void){printf("%%zu %%zu %%zu %%zu %%zu %%zu %%zu\\n", sizeof(cfd3d_config), sizeof(cfd3d_bc_patch),'
        ' sizeof(cfd3d_connection), sizeof(cfd3d_block_desc), offsetof(cfd3d_config, precision),'
        ' offsetof(cfd3d_config, kinf), offsetof(cfd3d_block_desc, con));return 0;}\n' % HEADER)
    exe = tmp_path / "l"
    subprocess.run([cc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    mine = [C.sizeof(abi.Config), C.sizeof(abi.BcPatch), C.sizeof(abi.Connection), C.sizeof(abi.BlockDesc),
            abi.Config.precision.offset, abi.Config.kinf.offset, abi.BlockDesc.con.offset]
    assert got == mine


def test_create_rejects_bad_config_without_gpu():
    c = cases.make("plain_small", scale=8)
    c["cfg"]["timemethod"] = 4
    with pytest.raises(native.Cfd3dError) as e:
        native.Engine(c)
    assert e.value.code == abi.ERR_ARG


def test_create_rejects_bad_descriptor_without_gpu():
    """descriptor validation runs before device selection, so it reports the bad descriptor
    on a host without a GPU as well"""
    c = cases.make("plain_small", scale=8)
    c["blocks"][0]["bc"].append((abi.BC_WALL, (2, 1, 1, 3, 5, 5)))  # not on a face
    with pytest.raises(native.Cfd3dError) as e:
        native.Engine(c)
    assert e.value.code == abi.ERR_DESCRIPTOR
    c = cases.make("plain_small", scale=8)
    b = c["blocks"][0]
    b["xyz"] = b["xyz"][:, :, :3].copy()   # 2 cells along i: fewer than the stencil needs
    b["imax"] = 3
    with pytest.raises(native.Cfd3dError) as e:
        native.Engine(c)
    assert e.value.code == abi.ERR_DESCRIPTOR
