"""Memory preflight on real bases, as the reference's tests/test_memory_preflight.py:87-160 on the GPU
backend: a budget is enforced before anything is allocated, the safety-adjusted requirement is
accepted exactly, cross and Nedelec assemblers and a cached assembler reached through asm check their
budgets, and the device memory that constructing an assembler and assembling with it takes stays
within the estimate."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
sk = pytest.importorskip("skfemntv_gb300")
from skfemntv_gb300.forms import ddot, grad  # noqa: E402


def _mesh():
    return sk.MeshTet.init_tensor(np.linspace(0.0, 1.0, 4), np.linspace(0.0, 1.0, 3), np.linspace(0.0, 1.0, 2))


def _basis(mesh, comp=1):
    return sk.Basis(mesh, sk.ElementVector(sk.ElementTetP1(), dim=comp))


def test_budget_rejects_before_construction_and_accepts_the_exact_requirement():
    b = _basis(_mesh(), comp=3)
    est = sk.estimate_bilinear_memory(b)
    with pytest.raises(sk.AssemblyMemoryBudgetError) as captured:
        sk.NativeBilinearForm(b, memory_limit_bytes=est.construction_peak_total_bytes_upper_bound)
    err = captured.value
    assert err.estimate == est and err.required_bytes > err.memory_limit_bytes
    assert err.largest_allocation in str(err) and "local_dofs=12x12" in str(err)

    b1 = _basis(_mesh())
    est1 = sk.estimate_bilinear_memory(b1)
    required = int(np.ceil(est1.construction_peak_total_bytes_upper_bound * 1.25))
    assert sk.NativeBilinearForm(b1, memory_limit_bytes=required).memory_estimate == est1


def test_cross_n1_and_cached_assemblers_check_budgets():
    m = _mesh()
    test_basis, trial_basis = _basis(m, comp=3), _basis(m)
    est = sk.estimate_bilinear_memory(test_basis, trial_basis)
    assert est.kind == "cross-bilinear" and (est.row_local_dofs, est.column_local_dofs) == (12, 4)
    with pytest.raises(sk.AssemblyMemoryBudgetError):
        sk.NativeCrossBilinearForm(test_basis, trial_basis,
                                   memory_limit_bytes=est.construction_peak_total_bytes_upper_bound)
    assert getattr(test_basis, "_tab", None) is None  # rejected before the tabulation was made
    with pytest.raises(ValueError, match="memory_safety_factor"):
        sk.NativeBilinearForm(test_basis, memory_limit_bytes=10 ** 9, memory_safety_factor=0.5)

    nb = sk.AffineTetN1Basis(m)
    n1 = sk.estimate_tet_n1_assembly_memory(nb)
    with pytest.raises(sk.AssemblyMemoryBudgetError):
        sk.TetN1Assembler(nb, memory_limit_bytes=n1.construction_peak_total_bytes_upper_bound)

    @sk.BilinearForm
    def form(u, v, _w):
        return ddot(grad(u), grad(v))

    b = _basis(_mesh())
    K = sk.asm(form, b)
    assert K.shape == (b.N, b.N)
    est = sk.estimate_bilinear_memory(b)  # the basis now holds its DOF map: the total is unchanged
    with pytest.raises(sk.AssemblyMemoryBudgetError):
        sk.asm(form, b, memory_limit_bytes=est.construction_peak_total_bytes_upper_bound)


def _device_bytes_used(make):
    """Device memory taken while what ``make`` returns is alive (torch's
    cached blocks released first, so new ones show)."""
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0 = torch.cuda.mem_get_info()[0]
    keep = make()
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    del keep
    return used


@pytest.mark.parametrize("per_point", [False, True])
def test_p2_tensor_device_memory_within_estimate(per_point):
    """P2 anisotropic diffusion on a 24^3 x 6 cube: device memory taken by the pattern, the values, the
    element matrices, coefficient staging and (per-point tensor) the tabulation, against the estimate's
    incremental bytes (which also count the host matrix)."""
    from skfemntv_gb300.assembly import NativeTensorForm

    m = sk.MeshTet2.from_mesh(sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, 25),) * 3))
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP2(), dim=1))
    E, Q = b._coefficient_shape
    est = sk.estimate_bilinear_memory(b)
    rng = np.random.default_rng(0)
    M = 0.1 * rng.standard_normal((E, 3, 3))
    A = np.moveaxis(np.einsum("eij,ekj->eik", M, M) + np.eye(3), (1, 2), (0, 1))
    A_pub = np.broadcast_to(A[..., None], (3, 3, E, Q))
    if per_point:
        A_pub = A_pub * (1.0 + 0.01 * rng.random((1, 1, E, Q)))

    def make():
        form = NativeTensorForm(b)
        return form, form.assemble(A_pub)

    used = _device_bytes_used(make)
    bound = est.construction_peak_incremental_bytes_upper_bound
    print(f"P2 24^3 per_point={per_point}: device {used / 2**20:.1f} MiB, estimate {bound / 2**20:.1f} MiB")
    assert used <= bound


def test_n1_device_memory_within_estimate():
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, 33),) * 3)
    nb = sk.AffineTetN1Basis(m)
    est = sk.estimate_tet_n1_assembly_memory(nb)
    mu = np.linspace(0.5, 1.5, m.nelements)[:, None]

    def make():
        a = sk.TetN1Assembler(nb)
        return a, a.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=mu)

    used = _device_bytes_used(make)
    bound = est.construction_peak_incremental_bytes_upper_bound
    print(f"N1 32^3: device {used / 2**20:.1f} MiB, estimate {bound / 2**20:.1f} MiB")
    assert used <= bound
