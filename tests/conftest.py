import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
C_ATOM = os.path.join(GOLDEN, "c_atom", "FCIDUMP")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as orc
    orc.build(ref=True)
    return orc


@pytest.fixture(scope="session")
def data_dir(tmp_path_factory):
    return str(tmp_path_factory.mktemp("shci_data"))


@pytest.fixture(scope="session")
def w1_fcidump(data_dir):
    from shci_gb300 import synthetic
    return synthetic.workload_fcidump(1, data_dir)


@pytest.fixture(scope="session")
def cr_fcidump(data_dir):
    """The reference's Cr-dimer FCIDUMP (38 orbitals, D-infinity-h), unpacked from the
    committed gzip copy."""
    import gzip
    path = os.path.join(data_dir, "cr_dimer_FCIDUMP")
    if not os.path.exists(path):
        with gzip.open(os.path.join(GOLDEN, "cr_dimer", "FCIDUMP.gz"), "rb") as f:
            data = f.read()
        with open(path, "wb") as g:
            g.write(data)
    return path


@pytest.fixture(scope="session")
def cr_pins():
    import json
    return json.load(open(os.path.join(GOLDEN, "cr_dimer_pins.json")))


@pytest.fixture(scope="session")
def c_atom_pins():
    import json
    return json.load(open(os.path.join(GOLDEN, "c_atom_pins.json")))
