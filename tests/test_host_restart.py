"""Restart files of the drop-in program against the reference's
(write_restart / read_restart, src/io_config.c:28-130).

The reference writes, in order: dr_max, dv_max (doubles), the box record
(box_info: vol, lx, ly, lz, min_size, cell_size as doubles, cell_x, cell_y,
cell_z, cell_type as ints; 64 bytes), the particle record (p_info: NN, Ncell;
8 bytes), the N x 4 configuration (id, x, y, z) and its generator's state.
The drop-in program keeps the first five blocks and writes its own stream
position (seed, sweep index, Widom calls, cluster moves: 4 x uint64) last.

Without a GPU: the reference's own files (tests/golden/host_ref/nvt_restart,
recorded by tests/golden/make_host_golden.py) have that layout, and the host
program's records have the reference's sizes.  On a GPU: the drop-in
program's files match the reference's block for block (byte for byte where
the chain does not enter: the records, and the whole lattice file at sweep
0), and a run continued from a restart file is the uninterrupted run, bit
for bit.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden", "host_ref", "nvt_restart")
INPUT = os.path.join(HERE, "golden", "host_inputs", "nvt_restart.dat")
N = 256
HEAD = 8 + 8 + 64 + 8  # dr_max, dv_max, box record, particle record


def parse(blob, tail):
    dr, dv = struct.unpack_from("<2d", blob, 0)
    box = struct.unpack_from("<6d4i", blob, 16)
    nn, ncell = struct.unpack_from("<2i", blob, 80)
    conf = np.frombuffer(blob, dtype="<f8", count=4 * nn, offset=HEAD).reshape(nn, 4)
    assert len(blob) == HEAD + 32 * nn + tail
    return dr, dv, box, (nn, ncell), conf


def test_reference_restart_layout():
    """The reference's files at sweeps 0, 100, 200: the records hold the
    input's values, the configuration its ids in order inside the box, and
    the last 5000 bytes its generator (624 words and a position)."""
    L = 4 * (4 / 0.7) ** (1 / 3)
    for name in ("restart_000.bin", "restart_100.bin", "restart_200.bin"):
        blob = open(os.path.join(GOLD, name), "rb").read()
        dr, dv, box, (nn, ncell), conf = parse(blob, 5000)
        assert (dr, dv) == (0.15, 0.001)
        vol, lx, ly, lz, min_size, cell_size, cx, cy, cz, ctype = box
        assert abs(lx - L) < 1e-12 and lx == ly == lz and (cx, cy, cz, ctype) == (4, 4, 4, 2)
        assert abs(vol - N / 0.7) < 1e-9
        assert nn == N
        assert np.array_equal(conf[:, 0], np.arange(N))
        assert np.all(conf[:, 1:] >= 0) and np.all(conf[:, 1:] <= lx)


def test_host_records_have_the_reference_sizes(tmp_path):
    """sizeof(host_box) and sizeof(host_pinfo) in the drop-in program equal
    the reference's box_info (64) and p_info (8) on this compiler."""
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "hsmc_host.h"\n'
                   'int main(void) { printf("%zu %zu\\n", sizeof(host_box), sizeof(host_pinfo)); return 0; }\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=gnu99", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "hsmc_gb300", "host"), str(src), "-o", str(exe)], check=True)
    assert subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split() == ["64", "8"]


def _run(exe, cwd, text):
    (cwd / "in.dat").write_text(text)
    r = subprocess.run([exe, "-i", "in.dat"], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.gpu
def test_restart_files_match_reference_and_continue_bit_exact(gpu_lib, tmp_path):
    from hsmc_gb300 import build

    exe = build.build_host()
    a = tmp_path / "a"
    a.mkdir()
    _run(exe, a, open(INPUT).read())
    names = sorted(f for f in os.listdir(a) if f.startswith("restart_"))
    assert names == sorted(f for f in os.listdir(GOLD) if f.startswith("restart_"))
    for name in names:
        ours = open(a / name, "rb").read()
        ref = open(os.path.join(GOLD, name), "rb").read()
        assert ours[:HEAD] == ref[:HEAD], name           # dr_max, dv_max, box and particle records
        _, _, _, _, conf = parse(ours, 32)               # our stream position: 4 x uint64
        assert np.array_equal(conf[:, 0], np.arange(N))
        seed, sweep_index, widom, cluster = struct.unpack_from("<4Q", ours, len(ours) - 32)
        assert seed == 11 and widom == 0 and cluster == 0
        assert sweep_index == int(name[8:11]) + 1        # the index of the next sweep
    # sweep 0: the lattice, byte for byte
    assert open(a / "restart_000.bin", "rb").read()[:HEAD + 32 * N] == \
        open(os.path.join(GOLD, "restart_000.bin"), "rb").read()[:HEAD + 32 * N]

    # continue from sweep 100 for another 100 sweeps: the uninterrupted run's file at 200
    b = tmp_path / "b"
    b.mkdir()
    shutil.copy(a / "restart_100.bin", b / "from.bin")
    text = open(INPUT).read().replace("sweep_eq 100", "sweep_eq 0").replace("sweep_stat 200", "sweep_stat 101")
    _run(exe, b, text + "restart_read 1 from.bin\n")
    cont = open(b / "restart_100.bin", "rb").read()
    full = open(a / "restart_200.bin", "rb").read()
    assert cont == full
