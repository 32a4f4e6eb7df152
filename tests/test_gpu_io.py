"""The batched result writer reading the result slab straight from device
memory (one strided device-to-host copy per file): the same bytes as the
per-CDP writer of the reference's Dumper::dumpResult."""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import capi, su
from test_su import _cdp_result_case

pytestmark = pytest.mark.gpu


def test_result_files_from_device_slab(tmp_path):
    torch = pytest.importorskip("torch")
    headers, slab = _cdp_result_case(tmp_path)
    d = torch.from_numpy(slab).cuda()
    paths = [str(tmp_path / f"d{r}.su") for r in range(3)]
    capi.write_result_files(slab, headers, paths, device_ptr=d.data_ptr())
    for r in range(3):
        ref = tmp_path / f"ref{r}.su"
        su.write_su(str(ref), headers, slab[:, r, :])
        assert (tmp_path / f"d{r}.su").read_bytes() == ref.read_bytes()
