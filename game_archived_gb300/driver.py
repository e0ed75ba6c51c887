"""The reference's time loop around manage_rkhevi (src/coordinator.c:291-324).

``run`` takes two callables with the reference's meaning --
``linear_combine(s0, s1, out, c0, c1)`` and ``manage_rkhevi(dt, t)`` -- so the
same loop drives the GPU library, the reference build or the oracle.
"""


def start(model, linear_combine):
    """state_new = state_old and the first-step flag (coordinator.c:291-299)."""
    linear_combine(model.state_old, model.state_old, model.state_new, 1.0, 0.0)
    model.config["totally_first_step_bool"] = 1


def step(model, linear_combine, manage_rkhevi, dt, t):
    """one pass of the time loop (coordinator.c:302-324)"""
    linear_combine(model.state_new, model.state_old, model.state_old, 1.0, 0.0)
    manage_rkhevi(dt, t)
    model.config["totally_first_step_bool"] = 0


def run(model, n_steps, dt, linear_combine, manage_rkhevi, t0=0.0, callback=None):
    start(model, linear_combine)
    t = t0
    for i in range(n_steps):
        step(model, linear_combine, manage_rkhevi, dt, t)
        t += dt
        if callback is not None:
            callback(i, model)
    return t
