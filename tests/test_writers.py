"""Result writers against the reference C++ driver's own output files of
data/cpp_test_run (stored verbatim in tests/golden/writer_golden.npz): the
written bytes must be identical.  Host-only code: runs without a GPU."""
import os

import numpy as np
import pytest

from am_ml_suite_gb300 import _native as nat

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def wg():
    return np.load(os.path.join(HERE, "golden", "writer_golden.npz"))


def _read(path):
    with open(path, "rb") as f:
        return f.read()


def test_density_npy_is_byte_identical(tmp_path, wg):
    ref = bytes(wg["npy"])
    p = tmp_path / "ref.npy"
    p.write_bytes(ref)
    rho = np.load(p)
    assert rho.shape == (30, 15, 20)
    out = tmp_path / "density_field.npy"
    nat.write_density_npy(str(out), rho, rho.shape)                       # z-fastest input
    assert _read(out) == ref
    xf = np.ascontiguousarray(rho.transpose(2, 1, 0)).ravel()            # x-fastest input
    nat.write_density_npy(str(out), xf, rho.shape, nat.LAYOUT_XFASTEST)
    assert _read(out) == ref
    assert np.array_equal(np.load(out), rho)


def test_history_csv_is_byte_identical(tmp_path, wg):
    ref = bytes(wg["history"])
    rows = np.loadtxt(ref.decode().splitlines()[1:], delimiter=",")
    out = tmp_path / "history.csv"
    # the reference printed its doubles with 6 significant digits; the printed
    # values round-trip through the same format
    nat.write_history_csv(str(out), rows[:, 1], rows[:, 2])
    assert _read(out) == ref


def test_metadata_json_is_byte_identical(tmp_path, wg):
    import json

    ref = bytes(wg["metadata"])
    m = json.loads(ref.decode())
    out = tmp_path / "metadata.json"
    nat.write_metadata_json(
        str(out), case_name=m["case"], mode=m["mode"], provenance=m["provenance"],
        resolution_mm=m["resolution_mm"], nx=m["domain_shape"][0], ny=m["domain_shape"][1],
        nz=m["domain_shape"][2], n_elements=m["n_elements"], n_design=m["n_design"], n_fixed=m["n_fixed"],
        n_void=m["n_void"], volume_fraction_target=m["volume_fraction_target"], has_history=1,
        volume_fraction_final=m["volume_fraction_final"], compliance_final=m["compliance_final"],
        iterations=m["iterations"], converged=int(m["converged"]), elapsed_time_s=m["elapsed_time_s"],
        threads=m["openmp_threads"], filter_radius=m["simp_config"]["filter_radius"],
        E_min=m["simp_config"]["E_min"], penalty=m["simp_config"]["penalty"],
        move_limit=m["simp_config"]["move_limit"])
    assert _read(out) == ref


def test_writer_errors(tmp_path):
    with pytest.raises(nat.AmError) as e:
        nat.write_density_npy(str(tmp_path / "no_such_dir" / "x.npy"), np.zeros(8), (2, 2, 2))
    assert e.value.name == "AM_ERR_INVALID_ARG"
    with pytest.raises(ValueError):
        nat.write_density_npy(str(tmp_path / "x.npy"), np.zeros(7), (2, 2, 2))
