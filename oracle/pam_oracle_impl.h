/*
 * Body of the CPU oracle, compiled twice by pam_oracle.c: once with R=float
 * (the reference's FP32 expression order, no FMA contraction) and once with
 * R=double (the FP64 evaluation every result is also compared against).
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this code;
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as
 * the checker.
 *
 * All arrays are row-major on the expanded grid [nz][nx] (nz = nz_abc,
 * nx = nx_abc of the reference).  Only cells in [4, nz-4) x [4, nx-4) are
 * ever updated; the outer four-cell frame stays zero, as in every reference
 * kernel (cpp/Modeling.cu:517, src/utils.py:404).
 */

#define IX(z, x) ((size_t)(z) * (size_t)nx + (size_t)(x))

/* 8th-order second derivative along x / z, reference term order
 * (cpp/Modeling.cu:521-531). */
static inline R SFX(d2x)(const R *U, size_t i)
{
    return C0 * U[i] + C1 * (U[i + 1] + U[i - 1]) + C2 * (U[i + 2] + U[i - 2])
         + C3 * (U[i + 3] + U[i - 3]) + C4 * (U[i + 4] + U[i - 4]);
}
static inline R SFX(d2z)(const R *U, size_t i, size_t s)
{
    return C0 * U[i] + C1 * (U[i + s] + U[i - s]) + C2 * (U[i + 2 * s] + U[i - 2 * s])
         + C3 * (U[i + 3 * s] + U[i - 3 * s]) + C4 * (U[i + 4 * s] + U[i - 4 * s]);
}
/* 8th-order first derivative (cpp/Modeling.cu:595-603). */
static inline R SFX(d1)(const R *U, size_t i, size_t s)
{
    return A1 * (U[i + s] - U[i - s]) + A2 * (U[i + 2 * s] - U[i - 2 * s])
         + A3 * (U[i + 3 * s] - U[i - 3 * s]) + A4 * (U[i + 4 * s] - U[i - 4 * s]);
}
/* 64-point cross derivative, reference term order (cpp/Modeling.cu:674-693). */
static inline R SFX(dxz)(const R *U, size_t i, size_t s)
{
    const R a[5] = {(R)0, A1, A2, A3, A4};
    R acc = (R)0;
    for (int ax = 1; ax <= 4; ax++)
        for (int az = 1; az <= 4; az++)
            acc = acc + a[ax] * a[az] * (U[i + az * s + ax] - U[i - az * s + ax]
                                        + U[i - az * s - ax] - U[i + az * s - ax]);
    return acc;
}

static inline int SFX(in_xstrip)(int x, int nx, int N) { return (x >= 4 && x < N) || (x >= nx - N && x < nx - 4); }
static inline int SFX(in_zstrip)(int z, int nz, int N) { return (z >= 4 && z < N) || (z >= nz - N && z < nz - 4); }

/*
 * Pseudo-acoustic Sd term shared by VTI and TTI (cpp/Modeling.cu:605-611).
 * The reference switches Sd on only when |den| > 1e-12.
 */
static inline R SFX(sd_term)(R eps, R del, R px, R pz)
{
    R px2 = px * px, pz2 = pz * pz;
    R num = (R)(-2.0) * (eps - del) * px2 * pz2;
    R den = ((R)1 + (R)2 * eps) * (px2 * px2) + (pz2 * pz2) + (R)2 * ((R)1 + del) * px2 * pz2;
    R sd = (R)0;
    if (FABS(den) > (R)1e-12) sd = num / den;
    return sd;
}

/* Cerjan factor of a cell: x then z, the order of cpp/Modeling.cu:535-550
 * and src/utils.py:382-391. */
static inline R SFX(cerjan_apply)(R v, const R *A, int z, int x, int nz, int nx, int N)
{
    if (x < N) v = v * A[x];
    if (x >= nx - N) v = v * A[nx - 1 - x];
    if (z < N) v = v * A[z];
    if (z >= nz - N) v = v * A[nz - 1 - z];
    return v;
}

/*
 * One forward time step.  Uf holds U(t-1) on entry and U(t+1) on exit; Uc
 * holds U(t) (source already injected).  approx: 0 acoustic, 1 VTI, 2 TTI.
 *
 * Cerjan (A != NULL): the update reads every neighbour of Uc before any cell
 * is damped, then damps Uf and Uc in the border.  This is the race-free
 * reading of the fused kernels cpp/Modeling.cu:499-749 and is exactly the
 * post-update damping of src/Modeling2D.py:338-341.
 *
 * CPML (psix != NULL): memory variables on the full grid, zero outside their
 * strips; the step updates psi then zeta from Uc (src/utils.py:242-377) and
 * adds d(psi)+zeta inside the strips (src/utils.py:768-1306).  The tilted
 * (TTI) variant has no reference counterpart; it applies the same stretched
 * first and second derivatives and leaves the cross derivative unstretched.
 */
void SFX(og_step)(int approx, int nz, int nx, int N, R dz, R dx, R dt,
                  R *Uf, R *Uc, const R *vp, const R *eps, const R *del, const R *theta,
                  const R *A,
                  R *psix, R *zetax, R *psiz, R *zetaz,
                  const R *ax_, const R *bx_, const R *az_, const R *bz_)
{
    const size_t s = (size_t)nx;
    const R inv_dx = (R)1 / dx, inv_dz = (R)1 / dz;
    const R inv_dx2 = (R)1 / (dx * dx), inv_dz2 = (R)1 / (dz * dz);
    const R inv_dxdz = (R)1 / (dx * dz);
    const R dt2 = dt * dt;
    const int cpml = (psix != NULL);

    if (cpml) {
        /* psi from Uc (src/utils.py:249-297) */
#pragma omp parallel for schedule(static)
        for (int z = 4; z < nz - 4; z++)
            for (int x = 4; x < nx - 4; x++) {
                size_t i = IX(z, x);
                if (SFX(in_xstrip)(x, nx, N)) psix[i] = ax_[i] * psix[i] + bx_[i] * (SFX(d1)(Uc, i, 1) * inv_dx);
                if (SFX(in_zstrip)(z, nz, N)) psiz[i] = az_[i] * psiz[i] + bz_[i] * (SFX(d1)(Uc, i, s) * inv_dz);
            }
        /* zeta from Uc and the new psi (src/utils.py:312-375) */
#pragma omp parallel for schedule(static)
        for (int z = 4; z < nz - 4; z++)
            for (int x = 4; x < nx - 4; x++) {
                size_t i = IX(z, x);
                if (SFX(in_xstrip)(x, nx, N))
                    zetax[i] = ax_[i] * zetax[i] + bx_[i] * (SFX(d2x)(Uc, i) * inv_dx2 + SFX(d1)(psix, i, 1) * inv_dx);
                if (SFX(in_zstrip)(z, nz, N))
                    zetaz[i] = az_[i] * zetaz[i] + bz_[i] * (SFX(d2z)(Uc, i, s) * inv_dz2 + SFX(d1)(psiz, i, s) * inv_dz);
            }
    }

#pragma omp parallel for schedule(static)
    for (int z = 4; z < nz - 4; z++) {
        for (int x = 4; x < nx - 4; x++) {
            size_t i = IX(z, x);
            R pxx = SFX(d2x)(Uc, i) * inv_dx2;
            R pzz = SFX(d2z)(Uc, i, s) * inv_dz2;
            R vp2 = vp[i] * vp[i];
            R xs = 0, zs = 0, dpx = 0, dpz = 0;
            if (cpml) {
                if (SFX(in_xstrip)(x, nx, N)) { xs = 1; dpx = SFX(d1)(psix, i, 1) * inv_dx; }
                if (SFX(in_zstrip)(z, nz, N)) { zs = 1; dpz = SFX(d1)(psiz, i, s) * inv_dz; }
            }
            R out;
            if (approx == 0) {
                if (!cpml) {
                    out = vp2 * dt2 * (pxx + pzz) + (R)2 * Uc[i] - Uf[i];
                } else {
                    R ex = xs != 0 ? dpx + zetax[i] : (R)0;
                    R ez = zs != 0 ? dpz + zetaz[i] : (R)0;
                    out = vp2 * dt2 * (pxx + pzz + ex + ez) + (R)2 * Uc[i] - Uf[i];
                }
            } else {
                R px = SFX(d1)(Uc, i, 1) * inv_dx;
                R pz = SFX(d1)(Uc, i, s) * inv_dz;
                R e = eps[i], d = del[i];
                R pxxe = pxx, pzze = pzz;
                if (cpml) {
                    if (xs != 0) { px = px + dpx; pxxe = pxx + dpx + zetax[i]; }
                    if (zs != 0) { pz = pz + dpz; pzze = pzz + dpz + zetaz[i]; }
                }
                if (approx == 1) {
                    R sd = SFX(sd_term)(e, d, px, pz);
                    out = (R)2 * Uc[i] - Uf[i] + vp2 * dt2 * (((R)1 + (R)2 * e) + sd) * pxxe
                        + vp2 * dt2 * ((R)1 + sd) * pzze;
                } else {
                    R pxz = SFX(dxz)(Uc, i, s) * inv_dxdz;
                    R th = theta[i];
                    R c = COS(th), sn = SIN(th);
                    R pxr = px * c - pz * sn;
                    R pzr = px * sn + pz * c;
                    R sd = SFX(sd_term)(e, d, pxr, pzr);
                    R c2 = c * c, s2 = sn * sn, sin2th = (R)2 * sn * c;
                    out = (R)2 * Uc[i] - Uf[i] + vp2 * dt2 * (((R)1 + (R)2 * e) * c2 + s2 + sd) * pxxe
                        + vp2 * dt2 * (((R)1 + (R)2 * e) * s2 + c2 + sd) * pzze
                        - (R)2 * e * vp2 * dt2 * sin2th * pxz;
                }
            }
            Uf[i] = out;
        }
    }

    if (A != NULL) {
#pragma omp parallel for schedule(static)
        for (int z = 4; z < nz - 4; z++)
            for (int x = 4; x < nx - 4; x++) {
                if (x >= N && x < nx - N && z >= N && z < nz - N) continue;
                size_t i = IX(z, x);
                Uf[i] = SFX(cerjan_apply)(Uf[i], A, z, x, nz, nx, N);
                Uc[i] = SFX(cerjan_apply)(Uc[i], A, z, x, nz, nx, N);
            }
    }
}

/*
 * Imaging-condition adjoint products for VTI (approx 1) and TTI (approx 2),
 * cpp/Migration.cu:573-666 and :757-861.  P is the source wavefield at the
 * same time step, Ub the receiver wavefield.  Writes the scratch fields
 * AU, BU, HU (TTI only), QCxU, QCzU on the full grid (zero outside the
 * update region).
 */
void SFX(og_adjoint_products)(int approx, int nz, int nx, R dz, R dx,
                              const R *Ub, const R *P, const R *eps, const R *del, const R *theta,
                              R *AU, R *BU, R *HU, R *QCxU, R *QCzU)
{
    const size_t s = (size_t)nx;
    const R inv_dx = (R)1 / dx, inv_dz = (R)1 / dz;
    const R inv_dx2 = (R)1 / (dx * dx), inv_dz2 = (R)1 / (dz * dz);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++) {
            size_t i = IX(z, x);
            AU[i] = 0; BU[i] = 0; QCxU[i] = 0; QCzU[i] = 0;
            if (HU) HU[i] = 0;
            if (!(x >= 4 && x < nx - 4 && z >= 4 && z < nz - 4)) continue;
            R pxx = SFX(d2x)(P, i) * inv_dx2;
            R pzz = SFX(d2z)(P, i, s) * inv_dz2;
            R px = SFX(d1)(P, i, 1) * inv_dx;
            R pz = SFX(d1)(P, i, s) * inv_dz;
            R e = eps[i], d = del[i];
            R Av, Bv, Hv = 0, Cx = 0, Cz = 0, sd = 0;
            if (approx == 1) {
                R px2 = px * px, pz2 = pz * pz, px4 = px2 * px2, pz4 = pz2 * pz2;
                R num = (R)(-2.0) * (e - d) * px2 * pz2;
                R den = ((R)1 + (R)2 * e) * px4 + pz4 + (R)2 * ((R)1 + d) * px2 * pz2;
                if (FABS(den) > (R)1e-12) {
                    sd = num / den;
                    R inv_den2 = (R)1 / (den * den);
                    R factor = (R)4 * (e - d) * (((R)1 + (R)2 * e) * px4 - pz4) * inv_den2;
                    Cx = factor * px * pz2;
                    Cz = -factor * px2 * pz;
                }
                Av = (R)1 + (R)2 * e + sd;
                Bv = (R)1 + sd;
            } else {
                R c = COS(theta[i]), sn = SIN(theta[i]);
                R xi = px * c - pz * sn, eta = px * sn + pz * c;
                R xi2 = xi * xi, eta2 = eta * eta, xi4 = xi2 * xi2, eta4 = eta2 * eta2;
                R num = (R)(-2.0) * (e - d) * xi2 * eta2;
                R den = ((R)1 + (R)2 * e) * xi4 + eta4 + (R)2 * ((R)1 + d) * xi2 * eta2;
                if (FABS(den) > (R)1e-12) {
                    sd = num / den;
                    R den2 = den * den;
                    R K = ((R)1 + (R)2 * e) * xi4 - eta4;
                    R factor = (R)4 * (e - d) * xi * eta * K / den2;
                    Cx = factor * pz;
                    Cz = -factor * px;
                }
                R cos2 = c * c, sin2 = sn * sn;
                Av = ((R)1 + (R)2 * e) * cos2 + sin2 + sd;
                Bv = ((R)1 + (R)2 * e) * sin2 + cos2 + sd;
                Hv = (R)2 * e * SIN((R)2 * theta[i]);
            }
            R Q = pxx + pzz;
            AU[i] = Av * Ub[i];
            BU[i] = Bv * Ub[i];
            if (HU) HU[i] = Hv * Ub[i];
            QCxU[i] = Q * Cx * Ub[i];
            QCzU[i] = Q * Cz * Ub[i];
        }
}

/*
 * One receiver-side (adjoint) step of RTM fused with the zero-lag imaging
 * condition, cpp/Migration.cu:504-571 (acoustic) and :668-755 / :863-973
 * (VTI / TTI, which consume og_adjoint_products).  image and ilum are the
 * interior [nz-2N][nx-2N]; they accumulate Ub*P and P*P.  Cerjan damping as
 * og_step.  For the acoustic CPML case pass psix.. (the receiver field keeps
 * its own memory variables) and A = NULL.
 */
void SFX(og_rtm_step)(int approx, int nz, int nx, int N, R dz, R dx, R dt,
                      R *Uf, R *Uc, const R *P, R *image, R *ilum,
                      const R *vp, const R *AU, const R *BU, const R *HU, const R *QCxU, const R *QCzU,
                      const R *A,
                      R *psix, R *zetax, R *psiz, R *zetaz,
                      const R *ax_, const R *bx_, const R *az_, const R *bz_)
{
    const size_t s = (size_t)nx;
    const int nxf = nx - 2 * N;
    /* imaging first: it reads Uc before any damping (cpp/Migration.cu:541-552) */
#pragma omp parallel for schedule(static)
    for (int z = N; z < nz - N; z++)
        for (int x = N; x < nx - N; x++) {
            size_t i = IX(z, x);
            size_t o = (size_t)(z - N) * (size_t)nxf + (size_t)(x - N);
            ilum[o] = ilum[o] + P[i] * P[i];
            image[o] = image[o] + Uc[i] * P[i];
        }
    if (approx == 0) {
        SFX(og_step)(0, nz, nx, N, dz, dx, dt, Uf, Uc, vp, NULL, NULL, NULL, A,
                     psix, zetax, psiz, zetaz, ax_, bx_, az_, bz_);
        return;
    }
    const R inv_dx = (R)1 / dx, inv_dz = (R)1 / dz;
    const R inv_dx2 = (R)1 / (dx * dx), inv_dz2 = (R)1 / (dz * dz);
    const R inv_dxdz = (R)1 / (dx * dz);
#pragma omp parallel for schedule(static)
    for (int z = 4; z < nz - 4; z++)
        for (int x = 4; x < nx - 4; x++) {
            size_t i = IX(z, x);
            R op = SFX(d2x)(AU, i) * inv_dx2 + SFX(d2z)(BU, i, s) * inv_dz2;
            if (approx == 2) op = op - SFX(dxz)(HU, i, s) * inv_dxdz;
            op = op - SFX(d1)(QCxU, i, 1) * inv_dx - SFX(d1)(QCzU, i, s) * inv_dz;
            R vp2dt2 = vp[i] * vp[i] * dt * dt;
            Uf[i] = (R)2 * Uc[i] - Uf[i] + vp2dt2 * op;
        }
    if (A != NULL) {
#pragma omp parallel for schedule(static)
        for (int z = 4; z < nz - 4; z++)
            for (int x = 4; x < nx - 4; x++) {
                if (x >= N && x < nx - N && z >= N && z < nz - N) continue;
                size_t i = IX(z, x);
                Uf[i] = SFX(cerjan_apply)(Uf[i], A, z, x, nz, nx, N);
                Uc[i] = SFX(cerjan_apply)(Uc[i], A, z, x, nz, nx, N);
            }
    }
}

/*
 * Exact discrete adjoint of og_step for the acoustic Cerjan scheme (no
 * reference counterpart: the reference reuses the forward operator).  With
 * D the Cerjan factor and k = vp^2 dt^2 the forward step is
 *   c(t+1) = D (2 c~(t) + k L c~(t) - D c~(t-1)),
 * so the adjoint variable obeys
 *   l(t) = 2 D l(t+1) + L(k D l(t+1)) - D^2 l(t+2) (+ D R^T r(t)).
 * Lf holds l(t+2) on entry and l(t) on exit, Lc holds l(t+1).
 */
void SFX(og_adjoint_exact_step)(int nz, int nx, int N, R dz, R dx, R dt,
                                R *Lf, const R *Lc, const R *vp, const R *A, R *work)
{
    const size_t s = (size_t)nx;
    const R inv_dx2 = (R)1 / (dx * dx), inv_dz2 = (R)1 / (dz * dz);
    const R dt2 = dt * dt;
    /* work = k D l(t+1) on the update region, zero elsewhere */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; z++)
        for (int x = 0; x < nx; x++) {
            size_t i = IX(z, x);
            R v = 0;
            if (x >= 4 && x < nx - 4 && z >= 4 && z < nz - 4) {
                v = Lc[i];
                if (A) v = SFX(cerjan_apply)(v, A, z, x, nz, nx, N);
                v = vp[i] * vp[i] * dt2 * v;
            }
            work[i] = v;
        }
#pragma omp parallel for schedule(static)
    for (int z = 4; z < nz - 4; z++)
        for (int x = 4; x < nx - 4; x++) {
            size_t i = IX(z, x);
            R dc = Lc[i], dp = Lf[i];
            if (A) {
                dc = SFX(cerjan_apply)(dc, A, z, x, nz, nx, N);
                dp = SFX(cerjan_apply)(SFX(cerjan_apply)(dp, A, z, x, nz, nx, N), A, z, x, nz, nx, N);
            }
            Lf[i] = (R)2 * dc + (SFX(d2x)(work, i) * inv_dx2 + SFX(d2z)(work, i, s) * inv_dz2) - dp;
        }
}

#undef IX
