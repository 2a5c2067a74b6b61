"""CPU tests of the C ABI boundary: the library loads, exports every entry
point that include/pelec_mol.h declares, and its structs have the layout the
ctypes mirror assumes.  No compute call needs a GPU here."""
import ctypes
import os
import re
import subprocess

import pytest

from pelec_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(pc_\w+)\s*\(", src, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from pelec_gb300 import build, mol

    build.build()
    return mol.library()


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("pc_mol_create", "pc_mol_destroy", "pc_mol_rhs_level", "pc_mol_last_status"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_strings(lib):
    assert lib.pc_mol_abi_version() == abi.PC_MOL_ABI_VERSION
    assert lib.pc_mol_error_string(abi.PC_ERR_UNSUPPORTED) == b"unsupported configuration"
    assert lib.pc_mol_error_string(12345) == b"unknown status code"


def test_null_arguments_are_rejected(lib):
    assert lib.pc_mol_create(None, None) == abi.PC_ERR_INVALID_ARGUMENT
    assert lib.pc_mol_last_status(None, None) == abi.PC_ERR_INVALID_ARGUMENT
    assert lib.pc_mol_rhs_level(None, None, 0, None, None) == abi.PC_ERR_INVALID_ARGUMENT


def test_struct_layout_matches_c(tmp_path):
    """sizeof/offsetof of the C structs equal the ctypes mirror's."""
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "pelec_mol.h"\n'
        "int main(void){\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(pc_mechanism), sizeof(pc_mol_config), sizeof(pc_array4),'
        " sizeof(pc_box_desc), sizeof(pc_mol_status));\n"
        'printf("%zu %zu %zu\\n", offsetof(pc_mol_config, mech), offsetof(pc_box_desc, rhs),'
        " offsetof(pc_mechanism, const_rhoD));\n"
        "return 0;}\n"
    )
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    got = [int(v) for v in out]
    want = [ctypes.sizeof(abi.PcMechanism), ctypes.sizeof(abi.PcMolConfig), ctypes.sizeof(abi.PcArray4),
            ctypes.sizeof(abi.PcBoxDesc), ctypes.sizeof(abi.PcMolStatus),
            abi.PcMolConfig.mech.offset, abi.PcBoxDesc.rhs.offset, abi.PcMechanism.const_rhoD.offset]
    assert got == want


def test_create_without_gpu_reports_no_device(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from pelec_gb300 import mechanism, problems

    cfg = problems.make_config(mechanism.gamma_law_single())
    h = ctypes.c_void_p()
    assert lib.pc_mol_create(ctypes.byref(h), ctypes.byref(cfg)) == abi.PC_ERR_NO_DEVICE


def test_product_does_not_import_oracle():
    """The shipped package never imports the oracle (test infrastructure)."""
    pkg = os.path.join(ROOT, "pelec_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "from oracle" not in text, f
                assert "pc_oracle" not in text, f


def test_tile_shapes_are_reported_without_a_gpu(lib):
    from pelec_gb300 import mol

    shapes = [mol.MOLOperator.tile_shape(t) for t in range(abi.PC_NUM_LAUNCH_CONFIGS)]
    assert shapes[: abi.PC_NUM_TILES] == [(8, 8, 4, 256), (8, 8, 8, 512), (16, 8, 4, 512), (8, 4, 4, 128)]
    # the persistent configurations run the same shapes
    assert shapes[abi.PC_LAUNCH_PERSISTENT:] == shapes[: abi.PC_NUM_TILES]
    out = (ctypes.c_int * 4)()
    assert lib.pc_mol_tile_shape(abi.PC_NUM_LAUNCH_CONFIGS, out) == abi.PC_ERR_INVALID_ARGUMENT
    assert lib.pc_mol_tile_shape(-1, out) == abi.PC_ERR_INVALID_ARGUMENT
    assert lib.pc_mol_set_tile(None, 0) == abi.PC_ERR_INVALID_ARGUMENT
    assert lib.pc_mol_autotune(None, None, 0, None, 1, None, None, 0, None) == abi.PC_ERR_INVALID_ARGUMENT
