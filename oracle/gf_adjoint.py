"""Oracle (test infrastructure only): FP64 tangent-linear and adjoint of the SingleLayerQG
ETDRK4 / FilteredETDRK4 and RK4 / FilteredRK4 steps, and the gradient of a final-time kinetic energy with respect to
the initial PV q0 and the topographic PV eta.

It differentiates the DISCRETE step of the restatement in gf_oracle.py exactly:
  * calcN! (src/singlelayerqg.jl:356-382, 443-451, constant U): dealias! sol in place,
    psi_hat = f q_hat (f = -1/K^2 or -1/(K^2 + 1/l^2), src/singlelayerqg.jl:484-490),
    u_hat = -i l psi_hat, v_hat = i kr psi_hat, q,u,v = irfft2(.), qe = q + eta,
    N = -i kr rfft2(u qe) - i l rfft2(v qe) - i kr U eta_hat;
    with U(y) (src/singlelayerqg.jl:395-432): u' = u + U, Qx = d(eta)/dx, Qy = d(eta)/dy - U_yy,
    N = -rfft2(u' Qx) - rfft2(v Qy) - i kr rfft2(u' q) - i l rfft2(v q);
  * the FourierFlows ETDRK4 and RK4 stage sequences (restated in gf_oracle.TimeStepper.step),
    in which every calcN! dealiases its input array in place, so that later uses of that array
    see the dealiased values (RK4: RHS_s = N(X_s) + L X_s at X_s = M(X1 + c_s dt RHS_{s-1}),
    X1 = M u, new = X1 + dt (RHS1/6 + RHS2/3 + RHS3/3 + RHS4/6)).
Inner products: spectral arrays are real vectors of (Re, Im) pairs over the STORED half
spectrum, <a, b> = Re sum conj(a) b; physical arrays the plain sum.  With them
  rfft2^T(X) = Re(nx ny ifft2(X placed in the half plane, zero elsewhere)),
  irfft2^T(x) = w rfft2(x) / (nx ny), w = 2 for interior kr columns, 1 for kr = 0 and Nyquist.
The loss is SingleLayerQG.kinetic_energy (src/singlelayerqg.jl:546-553): sum over the full
spectrum of K^2 |psi_hat|^2 / (2 (nx ny)^2).
"""
import numpy as np

import gf_oracle as O


def _w(grid):
    w = np.full(grid.nkr, 2.0)
    w[0] = 1.0
    if grid.nx % 2 == 0:
        w[-1] = 1.0
    return w


def rfft2_T(X, grid):
    """Transpose of the unnormalised r2c transform (half spectrum -> real field)."""
    full = np.zeros(X.shape[:-1] + (grid.nx,), dtype=np.complex128)
    full[..., : grid.nkr] = X
    return np.real(np.fft.ifft2(full, axes=(-2, -1))) * (grid.nx * grid.ny)


def irfft2_T(x, grid):
    """Transpose of the normalised c2r transform (real field -> half spectrum)."""
    return np.fft.rfft2(x, axes=(-2, -1)) * _w(grid) / (grid.nx * grid.ny)


class SLQGAdjoint:
    """Tangent-linear and adjoint of an oracle SingleLayerQG problem stepped with ETDRK4,
    FilteredETDRK4, RK4 or FilteredRK4, with a constant U or U(y) (additive forcing does not
    change the derivative)."""

    def __init__(self, prob):
        ts = prob.timestepper
        self.varying = not prob.U_is_number
        if self.varying:
            g = prob.grid
            self.Uf = prob.U                                               # (ny, nx)
            self.Qy0 = -O.irfft2(-g.l ** 2 * O.rfft2(self.Uf), g)          # -U_yy
        if ts.kind not in ("ETDRK4", "RK4"):
            raise NotImplementedError("the adjoint follows the ETDRK4 and RK4 stages")
        self.kind = ts.kind
        self.L, self.dt = prob.L, prob.clock.dt
        self.p, self.g = prob, prob.grid
        g = self.g
        self.U0 = 0.0 if self.varying else prob.U
        self.f = (-g.invKrsq if prob.ell is None else -1.0 / (g.Krsq + 1.0 / prob.ell ** 2))
        self.mask = np.ones((g.ny, g.nkr))
        O.dealias(self.mask, g)
        self.filter = ts.filter if getattr(ts, "filtered", False) else None
        if ts.kind == "ETDRK4":
            self.c = dict(e=ts.expLdt, e2=ts.expLdt2, z=ts.zeta, a=ts.alpha, b=ts.beta, g=ts.gamma)

    # -- calcN! without its dealias (the input is already dealiased) and its derivatives
    def _fields(self, X):
        g, f = self.g, self.f
        psih = f * X
        return O.irfft2(X, g), O.irfft2(-1j * g.l * psih, g), O.irfft2(1j * g.kr * psih, g)

    def _dx(self, x):
        return O.irfft2(1j * self.g.kr * O.rfft2(x), self.g)

    def _dy(self, x):
        return O.irfft2(1j * self.g.l * O.rfft2(x), self.g)

    def _dT(self, x, k):
        """transpose of x -> irfft2(i k rfft2(x)) (k = kr or l)"""
        g = self.g
        return rfft2_T(np.conj(1j * k) * irfft2_T(x, g), g)

    def N(self, X, eta):
        g = self.g
        q, u, v = self._fields(X)
        if self.varying:
            u = u + self.Uf
            Qx, Qy = self._dx(eta), self.Qy0 + self._dy(eta)
            return (-O.rfft2(u * Qx) - O.rfft2(v * Qy) - 1j * g.kr * O.rfft2(u * q)
                    - 1j * g.l * O.rfft2(v * q))
        qe = q + eta
        return (-1j * g.kr * O.rfft2(u * qe) - 1j * g.l * O.rfft2(v * qe)
                - 1j * g.kr * self.U0 * O.rfft2(eta))

    def N_tlm(self, X, eta, dX, deta):
        g = self.g
        q, u, v = self._fields(X)
        dq, du, dv = self._fields(dX)
        if self.varying:
            u = u + self.Uf
            Qx, Qy = self._dx(eta), self.Qy0 + self._dy(eta)
            dQx, dQy = self._dx(deta), self._dy(deta)
            return (-O.rfft2(du * Qx + u * dQx) - O.rfft2(dv * Qy + v * dQy)
                    - 1j * g.kr * O.rfft2(du * q + u * dq) - 1j * g.l * O.rfft2(dv * q + v * dq))
        qe, dqe = q + eta, dq + deta
        return (-1j * g.kr * O.rfft2(du * qe + u * dqe) - 1j * g.l * O.rfft2(dv * qe + v * dqe)
                - 1j * g.kr * self.U0 * O.rfft2(deta))

    def N_adj(self, X, eta, Nbar):
        """(Xbar, etabar) = J^T Nbar at (X, eta)."""
        g = self.g
        q, u, v = self._fields(X)
        if self.varying:
            u = u + self.Uf
            Qx, Qy = self._dx(eta), self.Qy0 + self._dy(eta)
            abar = rfft2_T(1j * g.kr * Nbar, g)
            bbar = rfft2_T(1j * g.l * Nbar, g)
            cbar = rfft2_T(-Nbar, g)
            qbar = abar * u + bbar * v
            ub, vb = irfft2_T(abar * q + cbar * Qx, g), irfft2_T(bbar * q + cbar * Qy, g)
            Xbar = irfft2_T(qbar, g) + self.f * (1j * g.l * ub - 1j * g.kr * vb)
            etabar = self._dT(cbar * u, g.kr) + self._dT(cbar * v, g.l)
            return Xbar, etabar
        qe = q + eta
        abar = rfft2_T(1j * g.kr * Nbar, g)
        bbar = rfft2_T(1j * g.l * Nbar, g)
        qbar = abar * u + bbar * v
        etabar = qbar + self.U0 * abar
        ub, vb = irfft2_T(abar * qe, g), irfft2_T(bbar * qe, g)
        Xbar = irfft2_T(qbar, g) + self.f * (1j * g.l * ub - 1j * g.kr * vb)
        return Xbar, etabar

    # -- RK4 (src: FourierFlows RK4 restated in gf_oracle.TimeStepper.step)
    def _rk4_step(self, u, eta):
        L, dt, M = self.L, self.dt, self.mask
        X1 = M * u
        R1 = self.N(X1, eta) + L * X1
        X2 = M * (X1 + dt / 2 * R1)
        R2 = self.N(X2, eta) + L * X2
        X3 = M * (X1 + dt / 2 * R2)
        R3 = self.N(X3, eta) + L * X3
        X4 = M * (X1 + dt * R3)
        R4 = self.N(X4, eta) + L * X4
        new = X1 + dt * (R1 / 6 + R2 / 3 + R3 / 3 + R4 / 6)
        if self.filter is not None:
            new = self.filter * new
        return new, (X1, X2, X3, X4)

    def _rk4_tlm(self, u, eta, du, deta):
        L, dt, M = self.L, self.dt, self.mask
        X1, X2, X3, X4 = self._rk4_step(u, eta)[1]
        dX1 = M * du
        dR1 = self.N_tlm(X1, eta, dX1, deta) + L * dX1
        dX2 = M * (dX1 + dt / 2 * dR1)
        dR2 = self.N_tlm(X2, eta, dX2, deta) + L * dX2
        dX3 = M * (dX1 + dt / 2 * dR2)
        dR3 = self.N_tlm(X3, eta, dX3, deta) + L * dX3
        dX4 = M * (dX1 + dt * dR3)
        dR4 = self.N_tlm(X4, eta, dX4, deta) + L * dX4
        dnew = dX1 + dt * (dR1 / 6 + dR2 / 3 + dR3 / 3 + dR4 / 6)
        if self.filter is not None:
            dnew = self.filter * dnew
        return dnew

    def _rk4_adj(self, u, eta, ubar_new):
        """the RK4 stages in reverse: Rbar_s is the cotangent of RHS_s, Y_s = M Xbar_s"""
        cL, dt, M = np.conj(self.L), self.dt, self.mask
        X1, X2, X3, X4 = self._rk4_step(u, eta)[1]
        ub = self.filter * ubar_new if self.filter is not None else ubar_new
        R4b = dt / 6 * ub
        Xb, eb4 = self.N_adj(X4, eta, R4b)
        Y = M * (Xb + cL * R4b)
        X1b = ub + Y
        R3b = dt / 3 * ub + dt * Y
        Xb, eb3 = self.N_adj(X3, eta, R3b)
        Y = M * (Xb + cL * R3b)
        X1b = X1b + Y
        R2b = dt / 3 * ub + dt / 2 * Y
        Xb, eb2 = self.N_adj(X2, eta, R2b)
        Y = M * (Xb + cL * R2b)
        X1b = X1b + Y
        R1b = dt / 6 * ub + dt / 2 * Y
        Xb, eb1 = self.N_adj(X1, eta, R1b)
        return M * (X1b + Xb + cL * R1b), eb1 + eb2 + eb3 + eb4

    # -- one step: forward, tangent-linear, adjoint
    def step(self, u, eta):
        if self.kind == "RK4":
            return self._rk4_step(u, eta)
        c, M = self.c, self.mask
        X1 = M * u
        N1 = self.N(X1, eta)
        XA = M * (c["e2"] * X1 + c["z"] * N1)
        N2 = self.N(XA, eta)
        XB = M * (c["e2"] * X1 + c["z"] * N2)
        N3 = self.N(XB, eta)
        XC = M * (c["e2"] * XA + c["z"] * (2 * N3 - N1))
        N4 = self.N(XC, eta)
        new = c["e"] * X1 + c["a"] * N1 + 2 * c["b"] * (N2 + N3) + c["g"] * N4
        if self.filter is not None:
            new = self.filter * new
        return new, (X1, XA, XB, XC)

    def step_tlm(self, u, eta, du, deta):
        if self.kind == "RK4":
            return self._rk4_tlm(u, eta, du, deta)
        c, M = self.c, self.mask
        (X1, XA, XB, XC) = self.step(u, eta)[1]
        dX1 = M * du
        dN1 = self.N_tlm(X1, eta, dX1, deta)
        dXA = M * (c["e2"] * dX1 + c["z"] * dN1)
        dN2 = self.N_tlm(XA, eta, dXA, deta)
        dXB = M * (c["e2"] * dX1 + c["z"] * dN2)
        dN3 = self.N_tlm(XB, eta, dXB, deta)
        dXC = M * (c["e2"] * dXA + c["z"] * (2 * dN3 - dN1))
        dN4 = self.N_tlm(XC, eta, dXC, deta)
        dnew = c["e"] * dX1 + c["a"] * dN1 + 2 * c["b"] * (dN2 + dN3) + c["g"] * dN4
        if self.filter is not None:
            dnew = self.filter * dnew
        return dnew

    def step_adj(self, u, eta, ubar_new):
        """(ubar, etabar contribution) of one step, the stages taken in reverse."""
        if self.kind == "RK4":
            return self._rk4_adj(u, eta, ubar_new)
        c, M = self.c, self.mask
        cj = {k: np.conj(v) for k, v in c.items()}
        X1, XA, XB, XC = self.step(u, eta)[1]
        ub = self.filter * ubar_new if self.filter is not None else ubar_new
        Xb, eb4 = self.N_adj(XC, eta, cj["g"] * ub)
        Cb = M * Xb
        N3b = 2 * cj["b"] * ub + 2 * cj["z"] * Cb
        N1b = cj["a"] * ub - cj["z"] * Cb
        XAb = cj["e2"] * Cb
        Xb, eb3 = self.N_adj(XB, eta, N3b)
        Bb = M * Xb
        X1b = cj["e"] * ub + cj["e2"] * Bb
        N2b = 2 * cj["b"] * ub + cj["z"] * Bb
        Xb, eb2 = self.N_adj(XA, eta, N2b)
        Ab = M * (XAb + Xb)
        X1b = X1b + cj["e2"] * Ab
        N1b = N1b + cj["z"] * Ab
        Xb, eb1 = self.N_adj(X1, eta, N1b)
        return M * (X1b + Xb), eb1 + eb2 + eb3 + eb4

    # -- loss and gradients
    def kinetic_energy(self, sol):
        g = self.g
        return float(np.sum(_w(g) * g.Krsq * np.abs(self.f * sol) ** 2)) / (2 * (g.nx * g.ny) ** 2)

    def kinetic_energy_grad(self, sol):
        g = self.g
        return _w(g) * g.Krsq * self.f ** 2 * sol / (g.nx * g.ny) ** 2

    def initial_state(self, q0):
        """set_q! (src/singlelayerqg.jl:519-534): sol = rfft2(q0), dealiased by updatevars!."""
        return self.mask * O.rfft2(q0)

    def loss(self, q0, eta, nsteps):
        u = self.initial_state(q0)
        for _ in range(nsteps):
            u = self.step(u, eta)[0]
        return self.kinetic_energy(u)

    def gradient(self, q0, eta, nsteps):
        """Loss and its gradients with respect to q0 and eta (every step state stored)."""
        us = [self.initial_state(q0)]
        for _ in range(nsteps):
            us.append(self.step(us[-1], eta)[0])
        ubar = self.kinetic_energy_grad(us[-1])
        etabar = np.zeros_like(eta)
        for n in range(nsteps - 1, -1, -1):
            ubar, eb = self.step_adj(us[n], eta, ubar)
            etabar += eb
        return self.kinetic_energy(us[-1]), self.initial_state_T(ubar), etabar

    def initial_state_T(self, ubar):
        """transpose of initial_state: the cotangent of q0"""
        return rfft2_T(self.mask * ubar, self.g)

    def directional_derivative(self, q0, eta, nsteps, dq0, deta):
        """dL along (dq0, deta) from the tangent-linear model."""
        u, du = self.initial_state(q0), self.initial_state(dq0)
        for _ in range(nsteps):
            du = self.step_tlm(u, eta, du, deta)
            u = self.step(u, eta)[0]
        return float(np.sum(np.real(np.conj(self.kinetic_energy_grad(u)) * du)))


class SQGAdjoint(SLQGAdjoint):
    """Tangent-linear and adjoint of an oracle SurfaceQG problem (src/surfaceqg.jl:257-297):
    the SingleLayerQG form with psi_hat = -psihfrombh b_hat (K^-1 coth(H K)), no topography and
    no mean flow; the loss is SurfaceQG.kinetic_energy, the cotangent of b0 has no k = 0 mode
    (set_b! removes it)."""

    def __init__(self, prob):
        ts = prob.timestepper
        if ts.kind not in ("ETDRK4", "RK4"):
            raise NotImplementedError("the adjoint follows the ETDRK4 and RK4 stages")
        self.varying = False
        self.kind = ts.kind
        self.L, self.dt = prob.L, prob.clock.dt
        self.p, self.g = prob, prob.grid
        g = self.g
        self.U0 = 0.0
        self.f = -prob.psihfrombh
        self.mask = np.ones((g.ny, g.nkr))
        O.dealias(self.mask, g)
        self.filter = ts.filter if getattr(ts, "filtered", False) else None
        if ts.kind == "ETDRK4":
            self.c = dict(e=ts.expLdt, e2=ts.expLdt2, z=ts.zeta, a=ts.alpha, b=ts.beta, g=ts.gamma)

    def initial_state(self, b0):
        bh = O.rfft2(b0)
        bh[0, 0] = 0
        return self.mask * bh

    def initial_state_T(self, ubar):
        ub = self.mask * ubar
        ub[0, 0] = 0
        return rfft2_T(ub, self.g)


class MLQGAdjoint(SLQGAdjoint):
    """Tangent-linear and adjoint of an oracle MultiLayerQG problem (src/multilayerqg.jl:651-731,
    the nonlinear calcN!) stepped with ETDRK4, FilteredETDRK4, RK4 or FilteredRK4, with respect
    to the initial PV of every layer and to the topography eta (which enters through the bottom
    layer's Qx = d(eta)/dx + ..., Qy = ... + d(eta)/dy; the mean flow is a parameter).
    Per layer j, with psi_hat = S^-1 q_hat (per wavenumber, src/multilayerqg.jl:495-509),
    u'_j = irfft(-i l psi_hat_j) + U_j(y), v_j = irfft(i kr psi_hat_j), q_j = irfft(q_hat_j):
      N_j = -rfft(u'_j Qx_j) - rfft(v_j Qy_j) - i kr rfft(u'_j q_j) - i l rfft(v_j q_j)
            (+ mu K^2 psi_hat_n in the bottom layer),
    and its transpose for Nbar: abar, bbar, cbar = rfft^T(i kr Nbar, i l Nbar, -Nbar),
      ubar = abar q + cbar Qx, vbar = bbar q + cbar Qy, qbar = abar u' + bbar v,
      psibar = i l irfft^T(ubar) - i kr irfft^T(vbar) (+ mu K^2 Nbar_n in the bottom layer),
      Xbar = irfft^T(qbar) + S^-T psibar,
      etabar = -d/dx(cbar_n u'_n) - d/dy(cbar_n v_n) (transposes of the spectral derivatives).
    The loss is the total kinetic energy sum_j KE_j of MultiLayerQG.energies
    (src/multilayerqg.jl:918-951)."""

    def __init__(self, prob):
        if prob.linear:
            raise NotImplementedError("the adjoint covers the nonlinear step")
        ts = prob.timestepper
        if ts.kind not in ("ETDRK4", "RK4"):
            raise NotImplementedError("the adjoint follows the ETDRK4 and RK4 stages")
        self.varying = False
        self.kind = ts.kind
        self.L, self.dt = prob.L, prob.clock.dt
        self.p, self.g = prob, prob.grid
        g = self.g
        self.n = prob.nlayers
        self.mask = np.ones((g.ny, g.nkr))
        O.dealias(self.mask, g)
        self.filter = ts.filter if getattr(ts, "filtered", False) else None
        if ts.kind == "ETDRK4":
            self.c = dict(e=ts.expLdt, e2=ts.expLdt2, z=ts.zeta, a=ts.alpha, b=ts.beta, g=ts.gamma)
        self.U = prob.Uy[:, :, None]
        # the PV gradients without the topography's share (added back for a given eta)
        self.Qx0, self.Qy0 = prob.Qx.copy(), prob.Qy.copy()
        self.Qx0[-1] -= self._dx(prob.eta)
        self.Qy0[-1] -= self._dy(prob.eta)
        self.mu = prob.mu
        self.Hw = np.asarray(prob.H, dtype=np.float64) / np.sum(prob.H) if self.n > 1 else np.ones(1)

    def _psi(self, X):
        if self.n == 1:
            return -self.g.invKrsq * X
        return np.einsum("yxij,jyx->iyx", self.p.Sinv, X)

    def _psiT(self, P):
        if self.n == 1:
            return -self.g.invKrsq * P
        return np.einsum("yxij,iyx->jyx", self.p.Sinv, P)

    def _fields(self, X):
        g = self.g
        psih = self._psi(X)
        return psih, O.irfft2(X, g), O.irfft2(-1j * g.l * psih, g), O.irfft2(1j * g.kr * psih, g)

    def _Q(self, eta):
        Qx, Qy = self.Qx0.copy(), self.Qy0.copy()
        Qx[-1] += self._dx(eta)
        Qy[-1] += self._dy(eta)
        return Qx, Qy

    def N(self, X, eta):
        g = self.g
        psih, q, u, v = self._fields(X)
        u = u + self.U
        Qx, Qy = self._Q(eta)
        N = (-O.rfft2(u * Qx) - O.rfft2(v * Qy) - 1j * g.kr * O.rfft2(u * q)
             - 1j * g.l * O.rfft2(v * q))
        N[-1] += self.mu * g.Krsq * psih[-1]
        return N

    def N_tlm(self, X, eta, dX, deta):
        g = self.g
        psih, q, u, v = self._fields(X)
        dpsih, dq, du, dv = self._fields(dX)
        u = u + self.U
        Qx, Qy = self._Q(eta)
        dN = (-O.rfft2(du * Qx) - O.rfft2(dv * Qy) - 1j * g.kr * O.rfft2(du * q + u * dq)
              - 1j * g.l * O.rfft2(dv * q + v * dq))
        dN[-1] -= O.rfft2(u[-1] * self._dx(deta)) + O.rfft2(v[-1] * self._dy(deta))
        dN[-1] += self.mu * g.Krsq * dpsih[-1]
        return dN

    def N_adj(self, X, eta, Nbar):
        g = self.g
        psih, q, u, v = self._fields(X)
        u = u + self.U
        abar = rfft2_T(1j * g.kr * Nbar, g)
        bbar = rfft2_T(1j * g.l * Nbar, g)
        cbar = rfft2_T(-Nbar, g)
        Qx, Qy = self._Q(eta)
        ub, vb = irfft2_T(abar * q + cbar * Qx, g), irfft2_T(bbar * q + cbar * Qy, g)
        qbar = abar * u + bbar * v
        psib = 1j * g.l * ub - 1j * g.kr * vb
        psib[-1] += self.mu * g.Krsq * Nbar[-1]
        etabar = self._dT(cbar[-1] * u[-1], g.kr) + self._dT(cbar[-1] * v[-1], g.l)
        return irfft2_T(qbar, g) + self._psiT(psib), etabar

    def kinetic_energy(self, sol):
        g = self.g
        a = _w(g) * g.Krsq * np.abs(self._psi(sol)) ** 2
        return float(np.sum(self.Hw[:, None, None] * a)) / (2 * (g.nx * g.ny) ** 2)

    def kinetic_energy_grad(self, sol):
        g = self.g
        return self._psiT(self.Hw[:, None, None] * _w(g) * g.Krsq * self._psi(sol)) / (g.nx * g.ny) ** 2

    def initial_state(self, q0):
        """set_q! (src/multilayerqg.jl:842-870): rfft of every layer, the k = 0 mode zeroed,
        dealiased by updatevars!"""
        qh = O.rfft2(q0)
        qh[..., 0, 0] = 0
        return self.mask * qh

    def initial_state_T(self, ubar):
        ub = self.mask * ubar
        ub[..., 0, 0] = 0
        return rfft2_T(ub, self.g)


def random_topography(grid, kmax, amp, seed):
    """Random Fourier modes |k| <= kmax (in units of 2 pi / Lx) with Philox complex-normal
    coefficients (tag 0x544F504F), scaled so that the field's maximum |eta| is amp."""
    K = np.sqrt(grid.Krsq) * grid.Lx / (2 * np.pi)
    z = O.complex_normal(grid.Krsq.size, seed, 0, 0x544F504F).reshape(grid.Krsq.shape)
    eh = np.where((K <= kmax) & (grid.Krsq > 0), z, 0)
    eta = O.irfft2(eh, grid)
    return amp * eta / np.max(np.abs(eta))
