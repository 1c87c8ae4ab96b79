"""Adjoint of the leapfrog (csg_adjoint_*) on the GPU.

Checks, on a small two-disk merger (stars only):
  * a frozen replay of the recorded run reproduces its loss bit for bit;
  * the checkpointed backward (segments recomputed) equals the backward over
    the recorded lists (to the rounding of the cells' atomic sums);
  * the gradient w.r.t. the initial state matches central finite differences
    of the frozen-list map (h = 1e-6) to 1e-4 relative, in Barnes-Hut and in
    direct-sum mode, and w.r.t. the three orbital parameters through the
    torch.autograd.Function of the harness. Relative to max(|directional
    derivative|, 1e-3 |gradient|): along a direction almost orthogonal to the
    gradient the difference quotient is limited by the loss's own rounding
    over h (about 1e-12 absolute here), not by the adjoint;
  * the Barnes-Hut adjoint points where the FP64 direct-sum adjoint does.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from adjoint_harness import MergerProblem, floored_errors, rel_errors  # noqa: E402
from cosmosim_gb300 import lib  # noqa: E402

SMALL = dict(n=2000, substeps=40, checkpoint_every=8, dt=2e-3)


@pytest.fixture(scope="module")
def tree():
    pr = MergerProblem(**SMALL)
    loss, gp, gx, gv = pr.gradients(record=True)
    yield pr, loss, gp, gx, gv
    pr.close()


def test_frozen_replay_reproduces_the_recorded_loss(tree):
    pr, loss, *_ = tree
    assert pr.frozen_loss(*pr.z0) == loss


def test_checkpointed_backward_equals_recorded(tree):
    pr, loss, gp, gx, gv = tree
    b = pr.ic.bodies(*pr.z0)
    loss2 = pr.adj.forward(b, pr.target, record=False)
    assert loss2 == loss
    gx2, gv2 = pr.adj.backward()
    for a, c in ((gx2, gx), (gv2, gv)):
        assert np.abs(a - c).max() <= 1e-11 * np.abs(c).max()
    pr.adj.forward(b, pr.target, record=True)  # restore the recorded run


def test_tree_adjoint_matches_finite_differences(tree):
    pr, loss, gp, gx, gv = tree
    gnorm = np.sqrt((gx ** 2).sum() + (gv ** 2).sum())
    err = floored_errors(pr.fd_directions(gx, gv, k=8), gnorm)
    assert max(err) <= 1e-4, err


def test_orbital_parameter_gradient_matches_finite_differences(tree):
    pr, loss, gp, gx, gv = tree
    assert np.all(np.isfinite(gp)) and np.any(gp != 0)
    err = rel_errors(pr.fd_params(gp))
    assert max(err) <= 1e-4, err


def test_direct_adjoint_matches_finite_differences():
    pr = MergerProblem(n=1000, substeps=20, checkpoint_every=5, mode=lib.ADJ_DIRECT)
    loss, gp, gx, gv = pr.gradients(record=False)
    gnorm = np.sqrt((gx ** 2).sum() + (gv ** 2).sum())
    err = floored_errors(pr.fd_directions(gx, gv, k=6, frozen=False), gnorm)
    pr.close()
    assert max(err) <= 1e-4, err


def test_tree_adjoint_close_to_direct_sum_adjoint():
    kw = dict(n=1500, substeps=20, checkpoint_every=5, theta=0.3)
    t = MergerProblem(**kw)
    d = MergerProblem(mode=lib.ADJ_DIRECT, **kw)
    _, _, tx, tv = t.gradients()
    _, _, dx, dv = d.gradients()
    a = np.concatenate([tx.ravel(), tv.ravel()])
    b = np.concatenate([dx.ravel(), dv.ravel()])
    t.close()
    d.close()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 0.05


def test_adjoint_at_the_benchmark_size():
    """The differentiable-merger configuration itself: 10,000 stars, 200
    substeps at dt 2e-3, checkpoints every 20. 32 random directions of the
    initial state and the three orbital parameters against central
    differences (h = 1e-6) of the frozen-list map, to 1e-4; the Barnes-Hut
    adjoint against the FP64 direct-sum adjoint of the same run (they differ
    by the tree's theta = 0.5 approximation, not by the adjoint: cosine)."""
    pr = MergerProblem()  # n=10000, substeps=200, dt=2e-3, checkpoint_every=20
    loss, gp, gx, gv = pr.gradients(record=True)
    gnorm = np.sqrt((gx ** 2).sum() + (gv ** 2).sum())
    err = floored_errors(pr.fd_directions(gx, gv, k=32, h=1e-6), gnorm)
    perr = rel_errors(pr.fd_params(gp, h=1e-6))
    pr.close()
    assert max(err) <= 1e-4, err
    assert max(perr) <= 1e-4, perr
    d = MergerProblem(mode=lib.ADJ_DIRECT)
    _, _, dx, dv = d.gradients(record=False)
    d.close()
    a = np.concatenate([gx.ravel(), gv.ravel()])
    b = np.concatenate([dx.ravel(), dv.ravel()])
    assert a @ b / (np.linalg.norm(a) * np.linalg.norm(b)) > 0.95
