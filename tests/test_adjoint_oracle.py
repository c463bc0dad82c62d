"""CPU pins of the gradient oracle (oracle/adjoint.py): the broadened
truncated-SVD adjoint against finite differences, the untruncated MPDO
gradient against autograd through the exact dense density-matrix simulator,
and the truncated MPDO gradient (chi and kappa binding) against complex128
central finite differences of the same evolution."""
import pytest
import torch

from oracle import adjoint as A, mpdo_oracle as O, dense_dm as D


def _fd_complex(loss, M, h=1e-6):
    """Central differences of a real function of a complex matrix, returned
    in torch's gradient convention dL/dRe + i dL/dIm."""
    g = torch.zeros_like(M)
    with torch.no_grad():
        for idx in range(M.numel()):
            for ph in (1, 1j):
                mp, mm = M.clone(), M.clone()
                mp.view(-1)[idx] += h * ph
                mm.view(-1)[idx] -= h * ph
                g.view(-1)[idx] += (loss(mp) - loss(mm)) / (2 * h) * ph
    return g


@pytest.mark.parametrize('m,n,k', [(6, 4, 2), (4, 7, 3), (5, 5, 5), (8, 3, 3)])
def test_truncated_svd_adjoint_matches_fd(m, n, k):
    g = torch.Generator().manual_seed(m * 100 + n * 10 + k)
    M = torch.randn(m, n, dtype=torch.complex128, generator=g)
    C = torch.randn(m, n, dtype=torch.complex128, generator=g)
    W = torch.randn(m, m, dtype=torch.complex128, generator=g)

    def loss(X):
        # gauge-invariant functions of the sqrt(S) split (Circuit.py:116-126)
        # and of the kappa pass's U.S (TNNOptimizer.py:188-194)
        u, s, vh, _ = O.svd_truncate(X, k, None)
        ss = torch.sqrt(s).to(X.dtype)
        left, right = u * ss[None], ss[:, None] * vh
        us = u * s.to(X.dtype)[None]
        return (torch.trace(left @ left.conj().T @ W).real + (right.conj().T @ right).abs().pow(2).sum()
                + (C.conj() * (left @ right)).sum().real + (us @ us.conj().T).abs().sum())

    X = M.clone().requires_grad_(True)
    loss(X).backward()
    fd = _fd_complex(loss, M)
    assert (X.grad - fd).abs().max() <= 1e-6 * fd.abs().max()


def test_forward_unchanged_by_gradient_tracking():
    ang = A.ansatz_angles(4, 2, seed=5)
    p = {'ry': torch.tensor(1e-3, dtype=torch.float64), 'cz': torch.tensor(1e-2, dtype=torch.float64)}
    e0 = A.energy(ang, p, chi=4, kappa=2)
    e1 = A.energy(ang.clone().requires_grad_(True), p, chi=4, kappa=2)
    assert abs(e0.item() - e1.item()) < 1e-13


def test_untruncated_gradient_matches_dense():
    # chi and kappa never bind: the MPDO gradient is that of the exact channel
    n, layers = 3, 1
    ang = A.ansatz_angles(n, layers, seed=1).requires_grad_(True)
    p = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True)
         for k, v in (('ry', 1e-3), ('rz', 2e-3), ('cz', 1e-2))}
    e = A.energy(ang, p, chi=16, kappa=16)
    e.backward()
    ang_d = ang.detach().clone().requires_grad_(True)
    p_d = {k: v.detach().clone().requires_grad_(True) for k, v in p.items()}
    rho = D.run(n, [op for op in A.ansatz_ops(ang_d, p_d) if op[0] != 'truncate'])
    e_d = A.ising_energy_dense(rho, n)
    e_d.backward()
    assert abs(e.item() - e_d.item()) < 1e-12
    torch.testing.assert_close(ang.grad, ang_d.grad, rtol=0, atol=1e-10)
    for k in p:
        assert abs(p[k].grad.item() - p_d[k].grad.item()) <= 1e-7 * max(1.0, abs(p_d[k].grad.item()))


def test_truncated_gradient_matches_central_fd():
    # n=5, two ansatz layers, chi=4 and kappa=2 both bind (discarded weight
    # ~1e-4 per bond).  Angles: central differences with h = 1e-4.  Noise
    # probabilities (1e-3 .. 1e-2): the kappa truncation makes the energy
    # curved on the scale of p itself, so their differences use h = 1e-5
    # (the h^2 error at h = 1e-4 is ~1e-4; at 1e-5 it is ~1e-6).
    n, layers, chi, kappa = 5, 2, 4, 2
    ang = A.ansatz_angles(n, layers, seed=2)
    p = {k: torch.tensor(v, dtype=torch.float64) for k, v in (('ry', 1e-3), ('rz', 2e-3), ('cz', 1e-2))}
    a1 = ang.clone().requires_grad_(True)
    p1 = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    A.energy(a1, p1, chi, kappa).backward()

    st = O.product_state([[1, 0]] * n, connected=True)
    O.evolve(st, A.ansatz_ops(ang, p), chi=chi, kappa=kappa, noisy=True)
    assert max(st.discarded) > 1e-5 and max(d[0] for d in st.dims()[1:]) == chi

    f = lambda: A.energy(ang, p, chi, kappa)  # noqa: E731
    (fd_ang,) = A.central_fd(f, [ang], h=1e-4)
    torch.testing.assert_close(a1.grad, fd_ang, rtol=0, atol=1e-7)
    fd_p = A.central_fd(f, [p[k] for k in p], h=1e-5)
    for k, fd in zip(p, fd_p):
        assert abs(p1[k].grad.item() - fd.item()) < 3e-6, (k, p1[k].grad.item(), fd.item())


def test_noiseless_truncated_gradient_matches_central_fd():
    # ideal circuit (no Kraus legs): only the chi sweep truncates
    n, layers, chi = 5, 2, 2
    ang = A.ansatz_angles(n, layers, seed=3)
    a1 = ang.clone().requires_grad_(True)
    A.energy(a1, None, chi, None).backward()
    (fd,) = A.central_fd(lambda: A.energy(ang, None, chi, None), [ang], h=1e-4)
    torch.testing.assert_close(a1.grad, fd, rtol=0, atol=1e-7)
