"""CPU-side checks of the C ABI: the library loads and exports every entry point include/sphgpu.h declares,
the ctypes mirror matches the header's struct layout, and invalid arguments are rejected on the host."""
import ctypes
import os
import re
import subprocess

import pytest

from opensph_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "sphgpu.h")


def declared_functions():
    text = open(HEADER).read()
    decl = r"^(?:sphgpu_status|int|const char\s*\*|void\s*\*)\s*(sphgpu_[a-z_]+)\s*\("
    names = sorted(set(re.findall(decl, text, flags=re.M)))
    assert len(names) >= 20
    return names


def _lib_path():
    if not os.path.exists(abi.LIBRARY_PATH):
        pytest.skip("libsphgpu.so is not built")
    return abi.LIBRARY_PATH


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib_path())
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version():
    lib = ctypes.CDLL(_lib_path())
    assert lib.sphgpu_abi_version() == 3


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "sphgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(sphgpu_material), sizeof(sphgpu_config),"
        " offsetof(sphgpu_config, gravity_constant), offsetof(sphgpu_config, precision),"
        " offsetof(sphgpu_material, damage_range), offsetof(sphgpu_config, courant_number));"
        "printf(\"%zu %zu\\n\", offsetof(sphgpu_config, restitution_normal), offsetof(sphgpu_config, max_bounces));"
        "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    got = [ctypes.sizeof(abi.Material), ctypes.sizeof(abi.Config), abi.Config.gravity_constant.offset,
           abi.Config.precision.offset, abi.Material.damage_range.offset, abi.Config.courant_number.offset,
           abi.Config.restitution_normal.offset, abi.Config.max_bounces.offset]
    assert [int(x) for x in out] == got


def test_create_rejects_invalid_settings_without_device():
    lib = ctypes.CDLL(_lib_path())
    lib.sphgpu_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    # NULL config
    assert lib.sphgpu_create(None, ctypes.byref(h)) == abi.ERR_ARGUMENT
    # no materials
    cfg, keep = abi.make_config(10, [abi.basalt()])
    cfg.material_count = 0
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_ARGUMENT
    # unsupported leaf size (one warp owns a leaf)
    cfg, keep = abi.make_config(10, [abi.basalt()], gravity_leaf_size=64)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    assert b"leaf" in lib.sphgpu_last_error(None)
    # unknown integrator
    cfg, keep = abi.make_config(10, [abi.basalt()], integrator=7)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    # negative gravity recomputation period
    cfg, keep = abi.make_config(10, [abi.basalt()], gravity_recomputation_period=-1.0)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_ARGUMENT
    assert not h.value


def test_create_rejects_invalid_nbody_settings_without_device():
    lib = ctypes.CDLL(_lib_path())
    lib.sphgpu_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    # the N-body solver is integrated by leap-frog only
    cfg, keep = abi.make_nbody_config(10, integrator=abi.INTEGRATOR_PREDICTOR_CORRECTOR)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    # self-gravity is its only force
    cfg, keep = abi.make_nbody_config(10, forces=abi.FORCE_PRESSURE | abi.FORCE_SELF_GRAVITY)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    # the Courant criterion needs sound speeds the N-body state does not have
    cfg, keep = abi.make_nbody_config(10, timestep_criteria=abi.CRITERION_COURANT)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    # unknown handlers
    cfg, keep = abi.make_nbody_config(10, collision_handler=9)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    cfg, keep = abi.make_nbody_config(10, overlap_handler=-1)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_UNSUPPORTED
    assert b"overlap" in lib.sphgpu_last_error(None)
    cfg, keep = abi.make_nbody_config(10, allowed_overlap=-0.5)
    assert lib.sphgpu_create(ctypes.byref(cfg), ctypes.byref(h)) == abi.ERR_ARGUMENT
    assert not h.value


def test_null_handle_calls_return_argument_error():
    lib = ctypes.CDLL(_lib_path())
    assert lib.sphgpu_collide(None, ctypes.c_double(1.0)) == abi.ERR_ARGUMENT
    assert lib.sphgpu_particle_count(None, None) == abi.ERR_ARGUMENT
    assert lib.sphgpu_integrate(None) == abi.ERR_ARGUMENT
    assert lib.sphgpu_step(None, 1) == abi.ERR_ARGUMENT
    assert lib.sphgpu_destroy(None) == abi.OK
