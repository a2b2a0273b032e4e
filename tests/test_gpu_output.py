"""ibmdem_output_async: the snapshot files equal the host writer's files for the
same state, although the caller steps on while they are written (the next step
waits only for the device-to-host copies, not for the formatting)."""
import numpy as np
import pytest

import cases
from ibmdem import api

pytestmark = pytest.mark.gpu


def make(gpu_lib, seed):
    p, parts, bodies, field = cases.contact_case(seed=seed)
    c = gpu_lib.Case(p, parts, bodies, field, device=0)
    c.InitializationDEM()
    return p, c


def test_async_snapshot_matches_host_writer(gpu_lib, tmp_path):
    p, a = make(gpu_lib, 4)
    a.step(2)
    (tmp_path / "async").mkdir()
    (tmp_path / "host").mkdir()
    a.output_async(tmp_path / "async" / "Particle_2_0.dat", tmp_path / "async", step=2)
    a.step(1)  # modifies the records the snapshot copies from
    a.output_async(None, tmp_path / "async", step=3)
    a.output_wait()
    a.close()

    p, b = make(gpu_lib, 4)
    b.step(2)
    parts, nl = b.get_parcels()
    api.write_tecplot_markers(tmp_path / "host" / "Particle_2_0.dat", parts[:nl])
    api.write_body_probes(tmp_path / "host", 2, b.get_bodies(), float(p["rhof"]))
    b.step(1)
    api.write_body_probes(tmp_path / "host", 3, b.get_bodies(), float(p["rhof"]))
    b.close()
    got = (tmp_path / "async" / "Particle_2_0.dat").read_bytes()
    want = (tmp_path / "host" / "Particle_2_0.dat").read_bytes()
    assert got == want
    files = sorted(f.name for f in (tmp_path / "host").glob("*.probe"))
    assert files and files == sorted(f.name for f in (tmp_path / "async").glob("*.probe"))
    for f in files:
        assert (tmp_path / "async" / f).read_bytes() == (tmp_path / "host" / f).read_bytes()
        assert len((tmp_path / "async" / f).read_text().splitlines()) == 2
