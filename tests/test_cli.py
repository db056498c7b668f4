"""The drop-in programs `uniform` and `amr`: output files in the reference's byte layout, stdout lines
in its formats, its exit codes and flag rules (src/tgv3d_uniform.cu:92-203, src/tgv3d_amr.cu:565-907).

The .vti/.vtp layout is checked with the readers' own access pattern (scripts/preview_tgv3d.py:21-42:
the extent from WholeExtent, "_" after <AppendedData, a UInt64 byte count, then little-endian Float32;
boxes as 8 ascii points each) plus the exact header text the reference writes.
"""
import os
import re
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "jp-solver_gb300", "bin")
HOST = os.path.join(ROOT, "jp-solver_gb300", "host")

HARNESS = r'''
#include "cli_common.h"
int main(int argc, char** argv) {
    const int N = 3, NP = N * N * N;
    std::vector<float> q(NP), s(NP), v(3 * NP);
    for (int i = 0; i < NP; ++i) { q[i] = 0.5f * i - 3.f; s[i] = 0.25f * i; }
    for (int i = 0; i < 3 * NP; ++i) v[i] = -0.125f * i;
    std::string d = argv[1];
    cli::write_vti(d + "/a.vti", q, s, v, N);
    cli::write_vti(d + "/b.vti", q, s, std::vector<float>(), N);
    std::vector<cli::Box> bs = {{0, 0, 0, 16, 1}, {8, 16, 24, 8, 2}};
    cli::write_boxes(d + "/c.vtp", bs);
    return 0;
}
'''


def header(n, with_vel):
    """The XML the reference writes before the appended data (src/tgv3d_uniform.cu:122-131,
    src/tgv3d_amr.cu:605-611)."""
    nb = 4 * n ** 3
    e = "0 %d 0 %d 0 %d" % (n - 1, n - 1, n - 1)
    lines = ['<?xml version="1.0"?>',
             '<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
             '  <ImageData WholeExtent="%s" Origin="0 0 0" Spacing="1 1 1">' % e,
             '    <Piece Extent="%s">' % e,
             '      <PointData Scalars="Q" Vectors="velocity">' if with_vel else '      <PointData Scalars="Q">',
             '        <DataArray type="Float32" Name="Q" format="appended" offset="0"/>',
             '        <DataArray type="Float32" Name="speed" format="appended" offset="%d"/>' % (8 + nb)]
    if with_vel:
        lines.append('        <DataArray type="Float32" Name="velocity" NumberOfComponents="3" format="appended" '
                     'offset="%d"/>' % (16 + 2 * nb))
    lines += ['      </PointData>', '    </Piece>', '  </ImageData>', '  <AppendedData encoding="raw">', '_']
    return ("\n".join(lines)).encode()


def read_appended(raw, count):
    """The arrays after "_", each a UInt64 byte count and Float32 payload (the readers' layout)."""
    a = raw.find(b"<AppendedData")
    pos = raw.find(b"_", a) + 1
    out = []
    for _ in range(count):
        (nb,) = struct.unpack_from("<Q", raw, pos)
        out.append(np.frombuffer(raw, dtype="<f4", count=nb // 4, offset=pos + 8))
        pos += 8 + nb
    assert raw[pos:] == b"\n  </AppendedData>\n</VTKFile>\n"
    return out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_vti_and_vtp_byte_layout(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", HOST, "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    subprocess.run([str(exe), str(tmp_path)], check=True)
    n, np3 = 3, 27
    q = 0.5 * np.arange(np3, dtype=np.float32) - 3
    s = 0.25 * np.arange(np3, dtype=np.float32)
    v = -0.125 * np.arange(3 * np3, dtype=np.float32)
    for name, with_vel in (("a.vti", True), ("b.vti", False)):
        raw = (tmp_path / name).read_bytes()
        assert raw.startswith(header(n, with_vel)), name
        assert int(re.search(rb'WholeExtent="0 (\d+)', raw).group(1)) + 1 == n
        arrays = read_appended(raw, 3 if with_vel else 2)
        np.testing.assert_array_equal(arrays[0], q)
        np.testing.assert_array_equal(arrays[1], s)
        if with_vel:
            np.testing.assert_array_equal(arrays[2], v)
    txt = (tmp_path / "c.vtp").read_text()
    assert txt.startswith('<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian">')
    assert '<Piece NumberOfPoints="16" NumberOfLines="24">' in txt
    pts = np.array(re.search(r'<Points>.*?format="ascii">(.*?)</DataArray>', txt, re.S).group(1).split(),
                   dtype=float).reshape(-1, 3)
    assert pts.shape == (16, 3)
    assert pts[:8].min(0).tolist() == [0, 0, 0] and pts[:8].max(0).tolist() == [16, 16, 16]
    assert pts[8:].min(0).tolist() == [8, 16, 24] and pts[8:].max(0).tolist() == [16, 24, 32]
    levels = re.search(r'Name="level" format="ascii">\n(.*?)</DataArray>', txt, re.S).group(1).split()
    assert levels == ["1"] * 8 + ["2"] * 8
    conn = re.search(r'Name="connectivity" format="ascii">\n(.*?)</DataArray>', txt, re.S).group(1).split()
    offs = re.search(r'Name="offsets" format="ascii">\n(.*?)</DataArray>', txt, re.S).group(1).split()
    assert len(conn) == 48 and offs[-1] == "48" and len(offs) == 24
    # every box edge joins two corners that differ in exactly one coordinate
    c = np.array(conn, dtype=int).reshape(-1, 2)
    assert all(np.count_nonzero(pts[a] != pts[b]) == 1 for a, b in c)


def program(name):
    p = os.path.join(BIN, name)
    if not os.path.exists(p):
        pytest.skip("programs not built")
    return p


def test_programs_exit_2_on_n_not_multiple_of_mb():
    # checked before any device work, as the reference does (src/tgv3d_uniform.cu:148)
    for name, extra in (("uniform", []), ("amr", ["--l1", "all"])):
        r = subprocess.run([program(name), "--n", "12"] + extra, capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and "N%MB" in r.stderr, (name, r.returncode, r.stderr)


SAMPLE_U = re.compile(r"^  t\*=\d+\.\d{3}  E/E0=\d\.\d{5}  enstrophy=\d\.\d{6}e[+-]\d\d  mass_drift=\d\.\d{2}e[+-]\d\d$")
SAMPLE_A = re.compile(r"^  t\*=\d+\.\d{3} E/E0=\d\.\d{5} enstrophy=\d\.\d{6}e[+-]\d\d mass_drift=\d\.\d{2}e[+-]\d\d$")


@pytest.mark.gpu
def test_uniform_program_stdout_and_frames(tmp_path):
    pre = str(tmp_path / "u")
    r = subprocess.run([program("uniform"), "--n", "16", "--re", "400", "--tstar", "0.6", "--vtk", pre, "--frames",
                        "3"], capture_output=True, text=True, timeout=120)
    assert r.returncode in (0, 1), r.stderr          # CHECK (1): no enstrophy peak this early
    lines = r.stdout.splitlines()
    assert re.match(r"^\[jp-solver uniform\] TGV3D N=16 MB=8 blocks=8 Re=400 nu=\S+ tau=0\.\d{4} steps=31 "
                    r"t\*max=0\.6  \(writing vti\)$", lines[0]), lines[0]
    samples = [l for l in lines if l.startswith("  t*=")]
    assert samples and all(SAMPLE_U.match(l) for l in samples), samples[:3]
    assert lines[-1].startswith("  wrote 3 vti frames")
    for k in range(3):
        raw = open("%s_%04d.vti" % (pre, k), "rb").read()
        assert raw.startswith(header(16, True))
        q, spd, vel = read_appended(raw, 3)
        assert q.size == 16 ** 3 and vel.size == 3 * 16 ** 3
        assert abs(float(spd.max()) - 0.05) < 0.01        # |u| of the TGV peaks at u0


@pytest.mark.gpu
def test_amr_program_stdout_and_frames(tmp_path):
    pre = str(tmp_path / "a")
    r = subprocess.run([program("amr"), "--n", "16", "--re", "800", "--tstar", "0.4", "--l1", "slab", "--l2", "all",
                        "--vtk", pre, "--frames", "2"], capture_output=True, text=True, timeout=120)
    assert r.returncode in (0, 1), r.stderr
    lines = r.stdout.splitlines()
    assert re.match(r"^\[jp-solver amr\] 3-level 3D\. N0=16 N1=32 N2=64 Re=800 L1=slab\(32 blk\) L2=all\(\d+ blk\) "
                    r"tau0=0\.\d{4} steps=\d+ \(vti\+vtp\)$", lines[0]), lines[0]
    samples = [l for l in lines if l.startswith("  t*=")]
    assert samples and all(SAMPLE_A.match(l) for l in samples), samples[:3]
    assert any(l.startswith("  pool high-water: L1 ") for l in lines)
    for k in range(2):
        raw = open("%s_%04d.vti" % (pre, k), "rb").read()
        assert raw.startswith(header(64, False))
        q, spd = read_appended(raw, 2)
        assert q.size == 64 ** 3
        txt = open("%s_%04d.vtp" % (pre, k)).read()
        m = re.search(r'NumberOfPoints="(\d+)" NumberOfLines="(\d+)"', txt)
        nbox = int(m.group(1)) // 8
        assert int(m.group(2)) == 12 * nbox and nbox >= 32          # 32 level-1 blocks + their level-2 children
