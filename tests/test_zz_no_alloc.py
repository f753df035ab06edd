"""The allocation-free k-space Ewald entry point (mg_ewald_kspace_noalloc).

Some callers cannot allocate device memory (a host that hands out all device
memory from its own pool, or a time-critical loop that cannot afford
cudaMalloc/cudaFree); this entry point keeps its scratch in a fixed array
inside the library.  The test calls it through the C ABI twice in a row, on
two different configurations, and checks each result against the context
entry point mg_ewald (same mixed-precision tolerance as the other tests).
It is collected last so that a failure here stops no other test."""
import ctypes as C

import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import load

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def test_noalloc_matches_context_entry_point_twice():
    import torch
    g, meta, system, ew = load("spce216")
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="mixed")
    lib = M.library()
    q = torch.tensor(system.q, dtype=torch.float64, device="cuda")
    Lb = np.ascontiguousarray(ew["L"], dtype=np.float64)
    for d in (0, 3):
        r = g["r"][d]
        fk, ek = fp.ewald(r)                      # the context entry point
        rd = torch.tensor(r.reshape(-1), dtype=torch.float64, device="cuda")
        fd = torch.full_like(rd, 7.0)             # overwritten by the call
        e = C.c_double()
        rc = lib.mg_ewald_kspace_noalloc(rd.data_ptr(), q.data_ptr(), system.ns,
                                         Lb.ctypes.data_as(C.POINTER(C.c_double)),
                                         ew["alpha"], ew["kappa"], fd.data_ptr(), C.byref(e),
                                         None)
        assert rc == 0
        f = fd.cpu().numpy().reshape(-1, 3)
        assert rel_rms(f, fk) < MIXED_TOL
        # energy on the Ewald energy scale (self term), as elsewhere
        eself = ew["alpha"] / np.sqrt(np.pi) * float((system.q ** 2).sum())
        assert abs(e.value - ek) < 2e-6 * eself


def test_noalloc_calls_leave_free_device_memory_unchanged():
    """The defining property: after a first call, further calls (also with
    another number of charges and another box) change the free device memory
    by nothing (cudaMemGetInfo, through torch)."""
    import torch
    lib = M.library()
    g, meta, system, ew = load("spce216")
    q = torch.tensor(system.q, dtype=torch.float64, device="cuda")
    r = torch.tensor(g["r"][0].reshape(-1), dtype=torch.float64, device="cuda")
    f = torch.zeros_like(r)
    e = C.c_double()
    L1 = np.ascontiguousarray(ew["L"], dtype=np.float64)
    L2 = L1 * 1.05

    def call(n, L):
        rc = lib.mg_ewald_kspace_noalloc(r.data_ptr(), q.data_ptr(), n,
                                         L.ctypes.data_as(C.POINTER(C.c_double)), ew["alpha"],
                                         ew["kappa"], f.data_ptr(), C.byref(e), None)
        assert rc == 0

    call(system.ns, L1)                       # warm-up: the module and its array are loaded
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for n, L in ((system.ns, L1), (system.ns - 90, L2), (300, L1), (system.ns, L2)):
        call(n, L)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    lib = M.library()
    n = 4097
    r = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    q = torch.ones(n, dtype=torch.float64, device="cuda")
    f = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    Lb = np.array([30.0, 30.0, 30.0])
    rc = lib.mg_ewald_kspace_noalloc(r.data_ptr(), q.data_ptr(), n,
                                     Lb.ctypes.data_as(C.POINTER(C.c_double)), 0.3, 0.2,
                                     f.data_ptr(), None, None)
    assert rc == 6   # MG_ERR_SIZE
    # too many k-vectors (|n| up to ~40 in a 30 A box)
    rc = lib.mg_ewald_kspace_noalloc(r.data_ptr(), q.data_ptr(), 100,
                                     Lb.ctypes.data_as(C.POINTER(C.c_double)), 0.3, 1.4,
                                     f.data_ptr(), None, None)
    assert rc == 6
