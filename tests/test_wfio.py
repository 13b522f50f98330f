"""Wavefunction checkpoints in the reference's "states" format (CPU): file
names and layout, the .occ file, round trips, and files made by the
reference's own FourierTransform (oracle/_ref) read back to the coefficients;
the transforms are the oracle's (the product passes its GPU plan instead)."""
import os
import shutil

import numpy as np
import pytest

from oracle import oracle as O
from qball_gb300 import synth
from qball_gb300 import wfio

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture()
def workdir():
    d = os.path.join(ROOT, "qball_gb300", "_build", "wfio_test")
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    yield d
    shutil.rmtree(d, ignore_errors=True)


@pytest.fixture(scope="module")
def states():
    cell = synth.make_cell("t12")
    a = np.diag([cell.L] * 3).reshape(9)
    b = O.Basis(a, cell.ecut)
    ft = O.FT(b, *b.np)
    c = synth.wavefunctions(cell, b, nst=3)
    return cell, a, b, ft, c


def test_file_names_follow_the_reference():
    assert wfio.state_file("wf", 7) == "wfk0000n00007"
    assert wfio.state_file("run/wf", 12, kp=3) == "run/wfk0003n00012"
    assert wfio.state_file("wf", 0, kp=1, spin=1) == "wfs1k0001n00000"
    assert wfio.occ_file("wf") == "wfk0000.occ"
    assert wfio.occ_file("wf", kp=2, spin=0) == "wfs0k0002.occ"


def test_round_trip_and_layout(states, workdir):
    cell, a, b, ft, c = states
    base = os.path.join(workdir, "wf")
    eig = np.array([-0.5, -0.25, 0.1])
    occ = np.array([2.0, 2.0, 0.0])
    names = wfio.write_states(base, c, ft.backward, eig=eig, occ=occ)
    N = int(np.prod(b.np))
    for n, name in enumerate(names):
        assert os.path.getsize(name) == 16 * N
        # the file is psi_n(r) on the basis grid, x fastest, no header
        assert np.array_equal(np.fromfile(name, np.complex128), ft.backward(c[n]))
    assert os.path.getsize(wfio.occ_file(base)) == 2 * 8 * 3
    c2, e2, o2 = wfio.read_states(base, 3, N, ft.forward, with_occ=True)
    assert np.abs(c2 - c).max() < 1e-13 * np.abs(c).max()
    assert np.array_equal(e2, eig) and np.array_equal(o2, occ)


def test_files_of_the_reference_transform(states, workdir):
    """States written through the reference's own FourierTransform::backward
    (compiled from its sources) are byte-identical to the restatement's and
    read back to the coefficients."""
    if O.ref() is None:
        pytest.skip("oracle/_ref not built")
    cell, a, b, ft, c = states
    rft = O.RefFT(a, cell.ecut, *b.np)
    base_r = os.path.join(workdir, "ref")
    base_o = os.path.join(workdir, "ora")
    wfio.write_states(base_r, c, rft.backward)
    wfio.write_states(base_o, c, ft.backward)
    for n in range(c.shape[0]):
        with open(wfio.state_file(base_r, n), "rb") as f1, open(wfio.state_file(base_o, n), "rb") as f2:
            assert f1.read() == f2.read()
    back = wfio.read_states(base_r, c.shape[0], int(np.prod(b.np)), rft.forward)
    assert np.abs(back - c).max() < 1e-13 * np.abs(c).max()


def test_missing_and_short_files(states, workdir):
    cell, a, b, ft, c = states
    base = os.path.join(workdir, "wf")
    N = int(np.prod(b.np))
    with pytest.raises(FileNotFoundError):
        wfio.read_states(base, 1, N, ft.forward)
    wfio.write_states(base, c[:1], ft.backward)
    with open(wfio.state_file(base, 0), "r+b") as fh:
        fh.truncate(16 * (N - 1))
    with pytest.raises(ValueError):
        wfio.read_states(base, 1, N, ft.forward)
    with pytest.raises(ValueError):
        wfio.write_states(base, c[:1], ft.backward, eig=[0.0])


@pytest.mark.gpu
def test_device_transforms_write_the_oracles_files(cuda, workdir, states):
    """The checkpoint files written through the C ABI's FP64 transforms (a
    plan on the basis' own grid) hold the oracle's psi(r) to 1e-13 and read
    back through the device forward transform to the coefficients."""
    import qball_gb300 as Q
    cell, a, b, ft, c = states
    qb = Q.Basis(a, cell.ecut)
    bwd, fwd = wfio.device_transforms(qb)
    base = os.path.join(workdir, "wf")
    wfio.write_states(base, c, bwd)
    n012 = int(np.prod(b.np))
    for n in range(c.shape[0]):
        f = np.fromfile(wfio.state_file(base, n), dtype=np.complex128)
        ref = ft.backward(c[n])
        assert np.linalg.norm(f - ref) <= 1e-13 * np.linalg.norm(ref)
    back = wfio.read_states(base, c.shape[0], n012, fwd)
    assert np.abs(back - c).max() < 1e-13
