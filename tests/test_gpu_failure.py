"""Failure detection of the cooperative field solvers, tested without a GPU
fault: one block of the solver's grid is told not to arrive at its grid
barriers and the waits give up after a short poll limit (a flag that nothing
sets, in the allowed form of a bounded wait).  The kernel must return, the
step must report MPG_ERR_TIMEOUT, and the context must stay usable: with the
test turned off the next step succeeds."""
import pytest

pytestmark = pytest.mark.gpu

FORMS = [("plain", "cg"), ("mixed", "cg"), ("mixed", "mg")]


@pytest.mark.parametrize("form,solver", FORMS)
def test_barrier_timeout_is_reported_and_ctx_recovers(mpg, form, solver):
    ctx = mpg.Ctx(0)
    ctx.mesh(16, split=mpg.SPLIT_KUHN6)
    ctx.configure(precision=mpg.PLAIN if form == "plain" else mpg.MIXED, deposit=mpg.DEPOSIT_LINEAR,
                  solver=mpg.SOLVER_CG_MG if solver == "mg" else mpg.SOLVER_CG, tol=1e-10, max_iter=5000,
                  warm_start=1, kill_on_wall=1, rho_background=1.0)
    n = 20000
    ctx.reserve(n)
    ctx.fill_uniform(n, 3, 0, 1.0 / n, vth=0.1)
    assert ctx.step(0.01, 1).rc == mpg.OK
    ctx.barrier_test(skip_block=1, poll_limit=1 << 14)
    st = ctx.step(0.01, 1, allow=(mpg.ERR_TIMEOUT,))
    assert st.rc == mpg.ERR_TIMEOUT
    assert "barrier" in ctx.last_error()
    ctx.barrier_test(-1)
    for _ in range(2):
        st = ctx.step(0.01, 1)
        assert st.rc == mpg.OK and st.solver_resid <= 1e-10
    assert 0 < ctx.count() <= n
