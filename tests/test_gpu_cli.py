"""The `nuray` executable (Cmd::main's argv grammar, src/cmd/cmd.cpp:9-114) on
a scene description written by the test: the Cornell box fixture as an OBJ
with an MTL file (Kd walls, Ke light). Its PNG / PFM / BMP outputs must hold
exactly what nr_render returns for the same scene text and parameters, and
renderer=nrc must run end to end with its cache."""
import os
import struct
import subprocess

import numpy as np
import pytest

import shim
from conftest import ROOT, golden

pytestmark = pytest.mark.gpu

PARAMS = ["renderer=ptnee", "imgw=64", "imgh=48", "spp=8", "campos=0,120,200", "cameuler=0,0,0", "camfov=64",
          "camasp=1.333"]


def write_cornell(d):
    g = golden("cornell_scene.npz")
    pos = g["pos"].reshape(-1, 3, 3)
    lines_mtl, lines_obj = [], ["mtllib box.mtl"]
    for i, (mi, mf) in enumerate(zip(g["mat_i"], g["mat_f"])):
        lines_mtl.append(f"newmtl m{i}")
        key = "Ke" if int(mi[0]) == 5 else "Kd"
        lines_mtl.append(f"{key} {mf[0]:.9g} {mf[1]:.9g} {mf[2]:.9g}")
    for k, (t, m) in enumerate(zip(pos, g["mat"])):
        lines_obj.append(f"usemtl m{int(m)}")
        for v in t:
            lines_obj.append(f"v {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}")
        lines_obj.append(f"f {3 * k + 1} {3 * k + 2} {3 * k + 3}")
    (d / "box.mtl").write_text("\n".join(lines_mtl) + "\n")
    (d / "box.obj").write_text("\n".join(lines_obj) + "\n")
    return str(d / "box.obj")


def run_cli(args):
    exe = os.path.join(ROOT, "nuray_gb300", "_build", "nuray")
    r = subprocess.run([exe, *args], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    return r.stdout


def read_pfm(path):
    data = open(path, "rb").read()
    head = data.split(b"\n", 3)
    w, h = (int(x) for x in head[1].split())
    scale = float(head[2])
    img = np.frombuffer(head[3], "<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return img[::-1]


def read_bmp(path):
    data = open(path, "rb").read()
    off, w, h = struct.unpack("<I", data[10:14])[0], struct.unpack("<i", data[18:22])[0], struct.unpack("<i", data[22:26])[0]
    row = (3 * w + 3) & ~3
    px = np.frombuffer(data[off:off + row * h], np.uint8).reshape(h, row)[:, :3 * w].reshape(h, w, 3)
    return px[::-1, :, ::-1]


def test_cli_outputs_equal_the_library(gpu_lib, tmp_path):
    from nuray_gb300 import Scene
    obj = write_cornell(tmp_path)
    out = run_cli([obj, "--output", str(tmp_path / "a.png"), "--params", *PARAMS])
    assert "finish" in out
    run_cli([obj, "--output", str(tmp_path / "a.pfm"), "--params", *PARAMS])
    run_cli([obj, "--output", str(tmp_path / "a.bmp"), "--params", *PARAMS])
    S = Scene.from_text(obj + "\n")
    hdr, rgb8 = S.render(" ".join(PARAMS), want_rgb8=True)
    np.testing.assert_array_equal(read_pfm(tmp_path / "a.pfm"), hdr)
    L = shim.load()
    png = shim.png_decode(L, (tmp_path / "a.png").read_bytes())
    np.testing.assert_array_equal(png[..., :3], rgb8)
    assert np.all(png[..., 3] == 255)
    np.testing.assert_array_equal(read_bmp(tmp_path / "a.bmp"), rgb8)


def test_cli_renderer_nrc(gpu_lib, tmp_path):
    obj = write_cornell(tmp_path)
    params = [p.replace("renderer=ptnee", "renderer=nrc") for p in PARAMS] + ["lr=0.001"]
    run_cli([obj, "--output", str(tmp_path / "n.pfm"), "--params", *params])
    img = read_pfm(tmp_path / "n.pfm")
    assert img.shape == (48, 64, 3) and np.all(np.isfinite(img)) and img.mean() > 0


def test_cli_rejects_unknown_renderer(gpu_lib, tmp_path):
    obj = write_cornell(tmp_path)
    exe = os.path.join(ROOT, "nuray_gb300", "_build", "nuray")
    r = subprocess.run([exe, obj, "--output", str(tmp_path / "x.png"), "--params", "renderer=bdpt", "imgw=4", "imgh=4"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 2 and "not available" in r.stdout
