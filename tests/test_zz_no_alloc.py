"""fcfcg_count_noalloc: unweighted counts for callers that cannot allocate
device memory (code inside another framework's memory pool, whose allocator
owns the device, or a program whose policy forbids cudaMalloc after
start-up).  Its results must equal those of the ordinary entry point,
fcfcg_count, call after call: the scratch it reuses between calls must not
leak one call's counts into the next.

This file is collected last on purpose; it passes alone and after the rest."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_counts(lib, host_ctx, ntot, a, b=None):
    import torch
    dev = torch.device("cuda", 0)
    cols_a = [torch.from_numpy(np.ascontiguousarray(a[:, k])).to(dev) for k in range(3)]
    if b is None:
        cols_b = [None, None, None]
        nb = 0
    else:
        cols_b = [torch.from_numpy(np.ascontiguousarray(b[:, k])).to(dev) for k in range(3)]
        nb = len(b)
    out = torch.full((ntot,), -1, dtype=torch.int64, device=dev)
    ptrs_b = [C.c_void_p(t.data_ptr()) if t is not None else None for t in cols_b]
    rc = lib.fcfcg_count_noalloc(host_ctx.h, int(b is None), len(a),
                                 *[C.c_void_p(t.data_ptr()) for t in cols_a],
                                 nb, *ptrs_b, C.c_void_p(out.data_ptr()), None)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_count_two_calls():
    import fcfc_gb300 as fg
    from fcfc_gb300 import synth
    lib = fg.load_library()

    # call 1: periodic box, (s, mu), clustered, auto
    box = 300.0
    kw = dict(box=box, smin=0, smax=40, ds=2.5, nmu=12)
    x = synth.neyman_scott(60, box, 40, 5.0, seed=7)
    host = fg.PairCounter("box", fg.BIN_SMU, host_only=True, **kw)
    dev = fg.PairCounter("box", fg.BIN_SMU, device=0, **kw)
    dev.load(0, x)
    want1 = dev.count_pairs(0)
    got1 = _noalloc_counts(lib, host, host.ntot, x)
    np.testing.assert_array_equal(got1, want1)
    assert want1.sum() > 0

    # call 2, same scratch: survey, (s_perp, pi) with log bins, cross
    kws = dict(ra=(150.0, 158.0), dec=(10.0, 17.0), zmu=0.5, zsig=0.04,
               zr=(0.46, 0.54))
    d = synth.radecz_to_xyz(synth.survey_radecz(2500, seed=8, **kws))
    r = synth.radecz_to_xyz(synth.survey_radecz(3000, seed=9, **kws))
    kw2 = dict(sedges=np.geomspace(0.5, 30, 11), pmin=0, pmax=30, dpi=3)
    host2 = fg.PairCounter("survey", fg.BIN_SPI, host_only=True, **kw2)
    dev2 = fg.PairCounter("survey", fg.BIN_SPI, device=0, **kw2)
    dev2.load(0, d)
    dev2.load(1, r)
    want2 = dev2.count_pairs(0, 1)
    got2 = _noalloc_counts(lib, host2, host2.ntot, d, r)
    np.testing.assert_array_equal(got2, want2)
    assert want2.sum() > 0

    # call 3: the first set-up again, nothing left over from call 2
    got3 = _noalloc_counts(lib, host, host.ntot, x)
    np.testing.assert_array_equal(got3, want1)


def test_noalloc_rejects_oversized_setup():
    import fcfc_gb300 as fg
    lib = fg.load_library()
    # 10000 x 255 bins of 8-byte accumulators exceed the 4 MiB scratch
    host = fg.PairCounter("survey", fg.BIN_SMU, host_only=True, smin=0,
                          smax=10000, ds=1, nmu=255)
    import torch
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(host.ntot, dtype=torch.int64, device="cuda")
    p = C.c_void_p(x.data_ptr())
    rc = lib.fcfcg_count_noalloc(host.h, 1, 4, p, p, p, 0, None, None, None,
                                 C.c_void_p(out.data_ptr()), None)
    assert rc == fg.capi.ERR_UNSUPPORTED
