"""The library's HDF5 reader on files in the reference's k-space layout
(MRI_DATA::write_external_data / read_external_data, src/mri_data.cpp:769-906), written
by tests/h5_writer.py with the HDF5 C++ library's default structures."""
import numpy as np
import pytest

from tests.h5_writer import write_mri_file
from tests.helpers import case, rel


def _encodes(nenc=2, C=3):
    out = []
    for e in range(nenc):
        c = case(N=16, C=C, nproj=40 + 10 * e, nread=16, seed=50 + e)
        shp = (1, 40 + 10 * e, 16)  # HDF5 order of the (readout, projections, slices) arrays
        out.append(dict(kx=c["kx"].reshape(shp), ky=c["ky"].reshape(shp), kz=c["kz"].reshape(shp),
                        kw=c["kw"].reshape(shp), kdata=c["data"].reshape((C,) + shp)))
    return out


def test_reader_reads_the_reference_layout(mrg_lib, tmp_path):
    enc = _encodes()
    path = tmp_path / "MRI_Raw.h5"
    write_mri_file(path, enc, 3)
    f = mrg_lib.H5File(path)
    assert f.attr_int("Kdata", "Num_Encodings") == 2
    assert f.attr_int("Kdata", "Num_Coils") == 3
    assert f.attr_int("/Kdata", "trajectory_typeX") == 1 and f.attr_int("Kdata", "dft_neededZ") == 1
    ne, nc, m = f.mri_info()
    assert (ne, nc, m) == (2, 3, [40 * 16, 50 * 16])
    for e in range(2):
        for key, name in (("kx", "KX_E%d"), ("ky", "KY_E%d"), ("kz", "KZ_E%d"), ("kw", "KW_E%d")):
            dims, cx = f.info("Kdata/" + name % e)
            assert dims == enc[e][key].shape and not cx
            assert np.array_equal(f.read("Kdata/" + name % e), enc[e][key])
        for c in range(3):
            d = f.read("/Kdata/KData_E%d_C%d" % (e, c))
            assert d.dtype == np.complex64 and np.array_equal(d, enc[e]["kdata"][c])
        assert f.read("Gating/TIME_E%d" % e).shape == enc[e]["kx"].shape[:-1]
        assert f.read("Gating/CLOCK_E%d" % e).shape == enc[e]["kx"].shape[:-1]


def test_reader_errors(mrg_lib, tmp_path):
    from mri_recon_gb300 import _lib
    path = tmp_path / "f.h5"
    write_mri_file(path, _encodes(1, 1), 1)
    f = mrg_lib.H5File(path)
    with pytest.raises(_lib.MrgError, match="not found"):
        f.read("Kdata/KX_E7")
    with pytest.raises(_lib.MrgError, match="attribute"):
        f.attr_int("Kdata", "Num_Frames")
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not hdf5 at all" * 100)
    with pytest.raises(_lib.MrgError, match="HDF5"):
        mrg_lib.H5File(bad)
    with pytest.raises(_lib.MrgError):
        mrg_lib.H5File(tmp_path / "missing.h5")


def test_reader_survives_damaged_files(mrg_lib, tmp_path):
    """Truncated files and files with corrupted bytes (header blocks, messages, sizes,
    addresses) either read or fail with MrgError: no crash, no read outside a message or
    the file, no allocation sized by a corrupted field."""
    import random
    from mri_recon_gb300 import _lib
    base = tmp_path / "base.h5"
    write_mri_file(base, _encodes(2, 2), 2)
    data = base.read_bytes()
    rng = random.Random(1234)
    path = tmp_path / "damaged.h5"
    outcomes = {"ok": 0, "error": 0}
    for i in range(400):
        b = bytearray(data)
        if i < 80:
            b = b[:rng.randrange(0, len(b))]
        else:
            for _ in range(rng.randint(1, 8)):
                pos = rng.randrange(0, 4096 if rng.random() < 0.7 else len(b))
                b[pos] = rng.randrange(256)
        path.write_bytes(bytes(b))
        try:
            f = mrg_lib.H5File(path)
            ne, nc, _ = f.mri_info()
            for e in range(min(ne, 4)):
                for name in ("KX_E%d", "KY_E%d", "KZ_E%d", "KW_E%d"):
                    f.read("Kdata/" + name % e)
                for c in range(min(nc, 4)):
                    f.read("Kdata/KData_E%d_C%d" % (e, c))
            outcomes["ok"] += 1
        except _lib.MrgError:
            outcomes["error"] += 1
    assert outcomes["error"] > 0 and outcomes["ok"] > 0, outcomes


@pytest.mark.gpu
def test_load_encode_into_a_plan(mrg_lib, tmp_path):
    """An encode loaded from the file through pinned memory into a plan frame gives the same
    E^H as the same arrays handed to the plan directly."""
    import torch
    enc = _encodes(2, 3)
    path = tmp_path / "MRI_Raw.h5"
    write_mri_file(path, enc, 3)
    f = mrg_lib.H5File(path)
    c = case(N=16, C=3, seed=9)
    p = mrg_lib.Plan(16, 3, 2)
    q = mrg_lib.Plan(16, 3, 2)
    for pl in (p, q):
        pl.set_smaps(torch.from_numpy(c["smaps"]).cuda())
    for e in range(2):
        f.load_encode(e, p, e)
        q.set_traj(e, *[enc[e][k].reshape(-1) for k in ("kx", "ky", "kz", "kw")])
        q.set_data(e, enc[e]["kdata"].reshape(3, -1))
    X1, _ = p.cg(2)
    X2, _ = q.cg(2)
    assert rel(X1.cpu().numpy(), X2.cpu().numpy()) < 1e-6
