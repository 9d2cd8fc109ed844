"""aar_gaussian_spectrum_noalloc: the Gaussian potential spectrum through the
C ABI with its seed-table scratch in static device memory, against the
plan-buffer path (aar_stage_noise + aar_copy_spectrum).  Collected last so it
also runs after every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest
import torch

from aarambam_gb300 import _lib
from aarambam_gb300.ic import ICGenerator
from tests.common import bbks, make_cfg, rel_rms, table

pytestmark = pytest.mark.gpu


def noalloc(g, out):
    stream = C.c_void_p(torch.cuda.current_stream(g.device).cuda_stream)
    return g.L.aar_gaussian_spectrum_noalloc(g.h, C.c_void_p(out.data_ptr()), stream)


@pytest.mark.parametrize("N,sphere,flip", [(64, 0, 0), (128, 1, 1)])
def test_noalloc_matches_plan_path_twice(cuda, N, sphere, flip):
    cfg = make_cfg(N, 500.0, 4321, 10.0, 8, "local_m8_L500_n128", max(N, 128), SphereMode=sphere, PhaseFlip=flip)
    g = ICGenerator(cfg, *table("local_m8_L500_n128", 8), *bbks())
    g.stage("noise")
    ref = g.spectrum()
    shape = (N, N, N // 2 + 1)
    outs = [torch.full(shape, complex(float("nan"), float("nan")), dtype=torch.complex64, device=cuda)
            for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for o in outs:  # two calls in a row
        assert noalloc(g, o) == _lib.AAR_OK, g.L.aar_last_error(g.h)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0  # no device memory taken
    assert g.L.aar_last_launch_count(g.h) == 2
    for o in outs:
        # same kernels on the same seed table: equal to the last bit
        torch.testing.assert_close(o, ref, rtol=0, atol=0)
    # the plan's own spectrum is untouched
    torch.testing.assert_close(g.spectrum(), ref, rtol=0, atol=0)


def test_noalloc_plain_form_matches_oracle(cuda):
    from oracle import oracle as O
    cfg = make_cfg(32, 500.0, 99, 10.0, 8, "local_m8_L500_n128", 128)
    k, t = bbks()
    g = ICGenerator(cfg, *table("local_m8_L500_n128", 8), k, t, precision="fp64")
    out = torch.empty((32, 32, 17), dtype=torch.complex128, device=cuda)
    for _ in range(2):
        assert noalloc(g, out) == _lib.AAR_OK, g.L.aar_last_error(g.h)
    w = O.Oracle(cfg, k, t).gauss()
    want = w[..., 0] + 1j * w[..., 1]
    got = out.cpu().numpy()
    assert np.array_equal(got == 0, want == 0)
    assert rel_rms(got, want) < 1e-12


def test_noalloc_rejects_oversized_grid(cuda):
    # plain FP64 plans go up to Nmesh 2048; the scratch holds Nmesh <= 1024
    cfg = make_cfg(1030, 500.0, 1, 10.0, 8, "local_m8_L500_n128", 1030)
    g = ICGenerator(cfg, *table("local_m8_L500_n128", 8), *bbks(), precision="fp64")
    out = torch.empty(16, dtype=torch.float64, device=cuda)
    assert noalloc(g, out) == _lib.AAR_ERR_ARG
    msg = g.L.aar_last_error(g.h).decode()
    assert "1030" in msg and "1024" in msg
