// Adjoint (forward with checkpoints / backward) of the fused step.
int Engine::forward(int nsteps, int ckpt) {
    (void)nsteps;
    (void)ckpt;
    return fail(VISG_ERR_UNSUPPORTED, "adjoint not available in this build");
}

int Engine::backward(const float*, const float*, float*, float*) {
    return fail(VISG_ERR_UNSUPPORTED, "adjoint not available in this build");
}
