"""The allocation-free FMM matvec (pibem_fmm_matvec_noalloc), for callers that
must not allocate device memory while they run (applications that reserve all
device memory up front, loops that cannot afford the synchronisation of
cudaMalloc / cudaFree).  Called through the C ABI with device buffers, twice in
a row (the second call finds the first call's contents in the shared scratch),
and compared with the allocating entry point pibem_fmm_matvec at the FP64
operator tolerance of the parity tests (1e-10 relative).  A request larger than
the fixed scratch is refused with PIBEM_EINVAL."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def test_noalloc_fmm_matvec_matches_allocating_entry_point(pibem_mod, synthetic):
    torch = pytest.importorskip("torch")
    mesh, mask, tmp, _ = synthetic.sphere_dirichlet_case(16)
    g = pibem_mod.BEMSolver(fma_truncation_order=4, max_nodes_per_childless_block=30)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    L = pibem_mod.load()
    n = mesh.n_nodes
    rng = np.random.Generator(np.random.PCG64(21))
    for call in range(2):
        phi = rng.normal(size=(2, n))
        dphi = rng.normal(size=(2, n))
        refN, refD = g.fmm_matvec(phi, dphi)
        dev = torch.device("cuda", 0)
        phi_d = torch.tensor(phi, device=dev, dtype=torch.float64)
        dphi_d = torch.tensor(dphi, device=dev, dtype=torch.float64)
        outN = torch.full((2, n), float("nan"), device=dev, dtype=torch.float64)
        outD = torch.full((2, n), float("nan"), device=dev, dtype=torch.float64)
        torch.cuda.synchronize()
        rc = L.pibem_fmm_matvec_noalloc(g.h, 2, C.c_void_p(phi_d.data_ptr()),
                                        C.c_void_p(dphi_d.data_ptr()), C.c_void_p(outN.data_ptr()),
                                        C.c_void_p(outD.data_ptr()))
        assert rc == pibem_mod.OK, L.pibem_last_error(g.h)
        torch.cuda.synchronize()
        assert rel(outN.cpu().numpy(), refN) < 1e-10
        assert rel(outD.cpu().numpy(), refD) < 1e-10
    # larger than the fixed scratch: refused, nothing launched
    rc = L.pibem_fmm_matvec_noalloc(g.h, 100000, C.c_void_p(phi_d.data_ptr()),
                                    C.c_void_p(dphi_d.data_ptr()), C.c_void_p(outN.data_ptr()),
                                    C.c_void_p(outD.data_ptr()))
    assert rc == pibem_mod.EINVAL
    assert b"MiB" in L.pibem_last_error(g.h)
    g.close()


def test_noalloc_fmm_matvec_float_float_mode(pibem_mod, synthetic):
    """In PIBEM_PRECISION_FLOAT_FLOAT mode pibem_fmm_matvec runs its translations
    in float-float arithmetic while the allocation-free call keeps the plain FP64
    far field: the two agree to the FP64-accurate operator tolerance (1e-11)."""
    torch = pytest.importorskip("torch")
    mesh, mask, tmp, _ = synthetic.sphere_dirichlet_case(16)
    g = pibem_mod.BEMSolver(fma_truncation_order=6, max_nodes_per_childless_block=30,
                            precision_mode=pibem_mod.PRECISION_FLOAT_FLOAT)
    g.set_mesh(mesh.xyz, mesh.cells)
    g.set_bc(mask)
    L = pibem_mod.load()
    n = mesh.n_nodes
    rng = np.random.Generator(np.random.PCG64(22))
    phi = rng.normal(size=n)
    dphi = rng.normal(size=n)
    refN, refD = g.fmm_matvec(phi, dphi)
    dev = torch.device("cuda", 0)
    phi_d = torch.tensor(phi, device=dev, dtype=torch.float64)
    dphi_d = torch.tensor(dphi, device=dev, dtype=torch.float64)
    outN = torch.empty(n, device=dev, dtype=torch.float64)
    outD = torch.empty(n, device=dev, dtype=torch.float64)
    torch.cuda.synchronize()
    rc = L.pibem_fmm_matvec_noalloc(g.h, 1, C.c_void_p(phi_d.data_ptr()),
                                    C.c_void_p(dphi_d.data_ptr()), C.c_void_p(outN.data_ptr()),
                                    C.c_void_p(outD.data_ptr()))
    assert rc == pibem_mod.OK, L.pibem_last_error(g.h)
    torch.cuda.synchronize()
    assert rel(outN.cpu().numpy(), refN.reshape(-1)) < 1e-11
    assert rel(outD.cpu().numpy(), refD.reshape(-1)) < 1e-11
    g.close()
