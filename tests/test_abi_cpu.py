"""CPU: the C-ABI shared library loads, exports every entry point that
include/pathtracer_gb300.h declares, its ctypes mirror has the C layout, and
calls fail cleanly (status codes, no crash) where there is no GPU."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from pathtracer_gb300 import native as N

REPO = Path(__file__).resolve().parents[1]
HEADER = REPO / "include" / "pathtracer_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^int (pt_[a-z_0-9]+)\(", text, flags=re.M)))


def test_header_and_binding_agree():
    assert sorted(N.EXPORTS) == declared_functions()


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N.LIB_PATH))
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version_without_gpu():
    assert N.load().pt_version() == 1


STRUCTS = {
    "pt_material_desc": N.MaterialDesc, "pt_mesh_desc": N.MeshDesc, "pt_quad_desc": N.QuadDesc,
    "pt_sphere_desc": N.SphereDesc, "pt_object_desc": N.ObjectDesc, "pt_env_desc": N.EnvDesc,
    "pt_medium_desc": N.MediumDesc, "pt_scene_desc": N.SceneDesc, "pt_camera_desc": N.CameraDesc,
    "pt_job_desc": N.JobDesc, "pt_stats": N.Stats, "pt_request_desc": N.RequestDesc,
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    lines = ['#include <stdio.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname in STRUCTS:
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
    lines.append('printf("job_camera %zu\\n", __builtin_offsetof(pt_job_desc, camera));')
    lines.append('printf("job_gamma %zu\\n", __builtin_offsetof(pt_job_desc, gamma));')
    lines.append('printf("scene_bg %zu\\n", __builtin_offsetof(pt_scene_desc, bg_color));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for cname, cls in STRUCTS.items():
        assert int(out[cname]) == C.sizeof(cls), cname
    assert int(out["job_camera"]) == N.JobDesc.camera.offset
    assert int(out["job_gamma"]) == N.JobDesc.gamma.offset
    assert int(out["scene_bg"]) == N.SceneDesc.bg_color.offset


def test_null_arguments_are_rejected():
    lib = N.load()
    assert lib.pt_create(None, 0) == -1  # PT_ERR_INVALID
    assert lib.pt_render(None, None, None, None) == -1
    assert lib.pt_scene_upload(None, None, None) == -1
    buf = C.create_string_buffer(128)
    assert lib.pt_last_error(None, buf, 128) == 0
    assert buf.value  # a message was recorded


def test_create_fails_cleanly_without_device():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = N.load()
    ctx = C.c_void_p()
    rc = lib.pt_create(C.byref(ctx), 0)
    assert rc == -2  # PT_ERR_CUDA, no crash
    buf = C.create_string_buffer(256)
    lib.pt_last_error(None, buf, 256)
    assert b"cuda" in buf.value.lower() or b"device" in buf.value.lower()
