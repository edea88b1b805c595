/*
 * ps_oracle_body.h -- type-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * Included twice by ps_oracle.c with REAL = double / float and SFX(name) = name_f64 / name_f32.
 */

#define OIDX(a, b, c, n) ((int64_t)(a) + (n)[0] * ((int64_t)(b) + (n)[1] * (int64_t)(c)))

/* Julia's Base.max / Base.min for IEEE floats (NaN-propagating, -0.0 < 0.0). */
static inline REAL SFX(jl_max)(REAL x, REAL y) {
    REAL diff = x - y;
    REAL r = signbit(diff) ? y : x;
    return (isnan(x) || isnan(y)) ? diff : r;
}
static inline REAL SFX(jl_min)(REAL x, REAL y) {
    REAL diff = x - y;
    REAL r = signbit(diff) ? x : y;
    return (isnan(x) || isnan(y)) ? diff : r;
}

/* Value of the FD macro {kind, opdims, inn} of A at thread index t
 * (src/FiniteDifferences.jl:54-61, 160-185, 328-394). */
static REAL SFX(fd_eval)(int kind, int opdims, int inn, int ndims, const REAL* A, const int64_t* nA,
                         const int64_t* t) {
    int64_t b[3];
    for (int d = 0; d < 3; d++) b[d] = t[d] + ((inn >> d) & 1);
    switch (kind) {
    case 0: /* selection */
        return A[OIDX(b[0], b[1], b[2], nA)];
    case 1: { /* A[i+1] - A[i] */
        int d = (opdims & 1) ? 0 : (opdims & 2) ? 1 : 2;
        int64_t p[3] = {b[0], b[1], b[2]};
        p[d] += 1;
        return A[OIDX(p[0], p[1], p[2], nA)] - A[OIDX(b[0], b[1], b[2], nA)];
    }
    case 2: { /* (A[i+1] - A[i]) - (A[i] - A[i-1]) */
        int d = (opdims & 1) ? 0 : (opdims & 2) ? 1 : 2;
        int64_t p[3] = {b[0], b[1], b[2]}, m[3] = {b[0], b[1], b[2]};
        p[d] += 1;
        m[d] -= 1;
        REAL c = A[OIDX(b[0], b[1], b[2], nA)];
        return (A[OIDX(p[0], p[1], p[2], nA)] - c) - (c - A[OIDX(m[0], m[1], m[2], nA)]);
    }
    case 3:   /* average: corners in x-fastest order, left-fold sum, times 0.5 / 0.25 / 0.125 */
    case 4: { /* harmonic: 1.0/(1.0/a + 1.0/b + ...)*k */
        int dims[3], k = 0;
        for (int d = 0; d < 3; d++)
            if ((opdims >> d) & 1) dims[k++] = d;
        int ncorner = 1 << k;
        REAL s = (REAL)0;
        for (int c = 0; c < ncorner; c++) {
            int64_t p[3] = {b[0], b[1], b[2]};
            for (int j = 0; j < k; j++) p[dims[j]] += (c >> j) & 1;
            REAL v = A[OIDX(p[0], p[1], p[2], nA)];
            if (kind == 4) v = (REAL)1.0 / v;
            s = (c == 0) ? v : s + v;
        }
        if (kind == 3) return s * ((REAL)1.0 / (REAL)ncorner);
        return ((REAL)1.0 / s) * (REAL)ncorner;
    }
    case 5:
    case 6: { /* maxloc / minloc: op(op(op(x-, x+), c), op(y-, y+)), ... */
        REAL m = 0;
        for (int d = 0; d < ndims; d++) {
            int64_t p[3] = {b[0], b[1], b[2]}, q[3] = {b[0], b[1], b[2]};
            p[d] -= 1;
            q[d] += 1;
            REAL lo = A[OIDX(p[0], p[1], p[2], nA)], hi = A[OIDX(q[0], q[1], q[2], nA)];
            REAL pair = (kind == 5) ? SFX(jl_max)(lo, hi) : SFX(jl_min)(lo, hi);
            if (d == 0) {
                REAL c = A[OIDX(b[0], b[1], b[2], nA)];
                m = (kind == 5) ? SFX(jl_max)(pair, c) : SFX(jl_min)(pair, c);
            } else {
                m = (kind == 5) ? SFX(jl_max)(m, pair) : SFX(jl_min)(m, pair);
            }
        }
        return m;
    }
    }
    return (REAL)0;
}

/* `@<lhs>(R) = @<op>(A)`: grid = max(size(R), size(A)); statement masked by `@within`
 * of the left-hand selection (lhs_inn), src/parallel.jl:654-680. */
int SFX(orc_fd_apply)(int kind, int opdims, int inn, int ndims, int lhs_inn, REAL* R, const int64_t* nR,
                      const REAL* A, const int64_t* nA) {
    int64_t lo[3], hi[3], tmax[3];
    for (int d = 0; d < 3; d++) {
        int li = (lhs_inn >> d) & 1;
        tmax[d] = nR[d] - 2 * li; /* threads passing the mask: 0 <= t < tmax */
        int rlo = 0, rhi = 0;
        if (kind == 1 || kind == 3 || kind == 4) rhi = (opdims >> d) & 1;
        if (kind == 2 || kind == 5 || kind == 6) rlo = rhi = (opdims >> d) & 1;
        lo[d] = ((inn >> d) & 1) - rlo;
        hi[d] = ((inn >> d) & 1) + rhi;
    }
    if (tmax[0] <= 0 || tmax[1] <= 0 || tmax[2] <= 0) return ORC_OK;
    for (int d = 0; d < 3; d++)
        if (lo[d] < 0 || tmax[d] - 1 + hi[d] > nA[d] - 1) return ORC_ERR_SHAPE;
    int lx = lhs_inn & 1, ly = (lhs_inn >> 1) & 1, lz = (lhs_inn >> 2) & 1;
#pragma omp parallel for schedule(static)
    for (int64_t tz = 0; tz < tmax[2]; tz++)
        for (int64_t ty = 0; ty < tmax[1]; ty++)
            for (int64_t tx = 0; tx < tmax[0]; tx++) {
                int64_t t[3] = {tx, ty, tz};
                R[OIDX(tx + lx, ty + ly, tz + lz, nR)] = SFX(fd_eval)(kind, opdims, inn, ndims, A, nA, t);
            }
    return ORC_OK;
}

/* `@all(T2) = @all(T) + @all(Ci)` over thread box [lo, hi) (examples/memcopy3D.jl:10-13). */
int SFX(orc_memcopy3d)(REAL* T2, const REAL* T, const REAL* Ci, const int64_t* n, const int64_t* lo,
                       const int64_t* hi) {
#pragma omp parallel for schedule(static)
    for (int64_t iz = lo[2]; iz < hi[2]; iz++)
        for (int64_t iy = lo[1]; iy < hi[1]; iy++)
            for (int64_t ix = lo[0]; ix < hi[0]; ix++) {
                int64_t i = OIDX(ix, iy, iz, n);
                T2[i] = T[i] + Ci[i];
            }
    return ORC_OK;
}

/* One step of the 3-D diffusion kernel in one of the four statement forms
 * (form 0: examples/diffusion3D_novis_noperf.jl:10-13; 1: examples/
 * diffusion3D_multigpucpu_hidecomm_novis.jl:12-15; 2: test/test_parallel.jl:420-426;
 * 3: the flux form with face conductivities @av_xi(lam) etc.). Thread box [lo, hi) of
 * the `@parallel` grid; the `@inn(T2)` mask gives cell c = t + 1 for t < n - 2. */
int SFX(orc_diffusion3d_step)(int form, REAL* T2, const REAL* T, const REAL* Ci, const REAL* lam_arr, REAL lam,
                              REAL dt, REAL hx, REAL hy, REAL hz, const int64_t* n, const int64_t* lo,
                              const int64_t* hi) {
    if (form < 0 || form > 3) return ORC_ERR_ARG;
    int64_t a[3], e[3];
    for (int d = 0; d < 3; d++) {
        a[d] = lo[d] < 0 ? 0 : lo[d];
        e[d] = hi[d] > n[d] - 2 ? n[d] - 2 : hi[d];
    }
    const int64_t sx = 1, sy = n[0], sz = n[0] * n[1];
#pragma omp parallel for schedule(static)
    for (int64_t tz = a[2]; tz < e[2]; tz++)
        for (int64_t ty = a[1]; ty < e[1]; ty++)
            for (int64_t tx = a[0]; tx < e[0]; tx++) {
                int64_t c = OIDX(tx + 1, ty + 1, tz + 1, n);
                REAL Tc = T[c];
                REAL out;
                if (form == 0 || form == 1) {
                    REAL d2x = (T[c + sx] - Tc) - (Tc - T[c - sx]);
                    REAL d2y = (T[c + sy] - Tc) - (Tc - T[c - sy]);
                    REAL d2z = (T[c + sz] - Tc) - (Tc - T[c - sz]);
                    REAL s;
                    if (form == 0)
                        s = (d2x / (hx * hx) + d2y / (hy * hy)) + d2z / (hz * hz);
                    else
                        s = (d2x * (hx * hx) + d2y * (hy * hy)) + d2z * (hz * hz);
                    out = Tc + dt * ((lam * Ci[c]) * s);
                } else {
                    REAL kxp, kxm, kyp, kym, kzp, kzm;
                    if (form == 2) {
                        kxp = kxm = kyp = kym = kzp = kzm = lam;
                    } else {
                        REAL lc = lam_arr[c];
                        kxp = (lc + lam_arr[c + sx]) * (REAL)0.5;
                        kxm = (lam_arr[c - sx] + lc) * (REAL)0.5;
                        kyp = (lc + lam_arr[c + sy]) * (REAL)0.5;
                        kym = (lam_arr[c - sy] + lc) * (REAL)0.5;
                        kzp = (lc + lam_arr[c + sz]) * (REAL)0.5;
                        kzm = (lam_arr[c - sz] + lc) * (REAL)0.5;
                    }
                    REAL qxp = ((-kxp) * (T[c + sx] - Tc)) * hx, qxm = ((-kxm) * (Tc - T[c - sx])) * hx;
                    REAL qyp = ((-kyp) * (T[c + sy] - Tc)) * hy, qym = ((-kym) * (Tc - T[c - sy])) * hy;
                    REAL qzp = ((-kzp) * (T[c + sz] - Tc)) * hz, qzm = ((-kzm) * (Tc - T[c - sz])) * hz;
                    REAL dTdt = Ci[c] * (((-(qxp - qxm)) * hx - (qyp - qym) * hy) - (qzp - qzm) * hz);
                    out = Tc + dt * dTdt;
                }
                T2[c] = out;
            }
    return ORC_OK;
}

/* Adjoint of one flux-form diffusion step with a conductivity array (form 3 above).
 * Forward: T2[c] = T[c] + dt*Ci[c]*Σ_d h_d*(-(q_d+ - q_d-)), q_d± the face fluxes with face
 * conductivity (lam_a + lam_b)*0.5, for inner cells c; boundary cells are fixed values.
 * Given lamT2 = ∂L/∂T2 (ignored on boundary cells), with μ = dt*Ci*lamT2 on inner cells and 0
 * elsewhere:
 *   lamT[c]  = lamT2[c] + Σ_d h_d² (k_d+(μ[c+e] - μ[c]) - k_d-(μ[c] - μ[c-e]))   (inner c; 0 else)
 *   glam[c] += 0.5 Σ_{faces (a, b=a+e) of c} (μ[a] - μ[b]) h_d² (T[b] - T[a])   (all cells)
 * This is the transpose of the forward step's Jacobian (the operator is symmetric in T). */
int SFX(orc_diffusion3d_adjoint_step)(REAL* lamT, const REAL* lamT2, const REAL* T, const REAL* Ci, const REAL* lam,
                                      REAL* glam, REAL dt, REAL hx, REAL hy, REAL hz, const int64_t* n) {
    const int64_t nx = n[0], ny = n[1], nz = n[2], sy = nx, sz = nx * ny;
    const REAL hh[3] = {hx * hx, hy * hy, hz * hz};
    const int64_t st[3] = {1, sy, sz};
#define INNER(i, j, k) ((i) >= 1 && (i) <= nx - 2 && (j) >= 1 && (j) <= ny - 2 && (k) >= 1 && (k) <= nz - 2)
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nz; k++)
        for (int64_t j = 0; j < ny; j++)
            for (int64_t i = 0; i < nx; i++) {
                const int64_t c = OIDX(i, j, k, n);
                const int64_t idx[3] = {i, j, k}, ext[3] = {nx, ny, nz};
                const int inner_c = INNER(i, j, k);
                const REAL mu_c = inner_c ? dt * Ci[c] * lamT2[c] : (REAL)0;
                REAL acc = (REAL)0, g = (REAL)0;
                for (int d = 0; d < 3; d++) {
                    for (int sgn = -1; sgn <= 1; sgn += 2) {
                        const int64_t q = idx[d] + sgn;
                        if (q < 0 || q >= ext[d]) continue;
                        int64_t ii = i, jj = j, kk = k;
                        if (d == 0) ii = q;
                        if (d == 1) jj = q;
                        if (d == 2) kk = q;
                        const int64_t nb = c + sgn * st[d];
                        const REAL mu_n = INNER(ii, jj, kk) ? dt * Ci[nb] * lamT2[nb] : (REAL)0;
                        const REAL kf = (lam[c] + lam[nb]) * (REAL)0.5;
                        /* face (a, b) with a the lower cell */
                        const REAL mua = sgn > 0 ? mu_c : mu_n, mub = sgn > 0 ? mu_n : mu_c;
                        const REAL Ta = sgn > 0 ? T[c] : T[nb], Tb = sgn > 0 ? T[nb] : T[c];
                        acc += hh[d] * kf * (mu_n - mu_c);
                        g += (REAL)0.5 * (mua - mub) * hh[d] * (Tb - Ta);
                    }
                }
                lamT[c] = inner_c ? lamT2[c] + acc : (REAL)0;
                glam[c] += g;
            }
#undef INNER
    return ORC_OK;
}

/* acoustic3D compute_V! (miniapps/acoustic3D.jl:11-16): grid (nx+1, ny+1, nz+1);
 * P is (nx, ny, nz), Vx (nx+1, ny, nz), Vy (nx, ny+1, nz), Vz (nx, ny, nz+1). */
int SFX(orc_acoustic3d_v)(REAL* Vx, REAL* Vy, REAL* Vz, const REAL* P, const int64_t* n, REAL dt, REAL rho,
                          REAL dx, REAL dy, REAL dz) {
    int64_t nx = n[0], ny = n[1], nz = n[2];
    int64_t nVx[3] = {nx + 1, ny, nz}, nVy[3] = {nx, ny + 1, nz}, nVz[3] = {nx, ny, nz + 1};
    REAL dtr = dt / rho;
#pragma omp parallel for schedule(static)
    for (int64_t tz = 0; tz < nz + 1; tz++)
        for (int64_t ty = 0; ty < ny + 1; ty++)
            for (int64_t tx = 0; tx < nx + 1; tx++) {
                if (tx < nVx[0] - 2 && ty < nVx[1] - 2 && tz < nVx[2] - 2) {
                    int64_t v = OIDX(tx + 1, ty + 1, tz + 1, nVx);
                    REAL d = P[OIDX(tx + 1, ty + 1, tz + 1, n)] - P[OIDX(tx, ty + 1, tz + 1, n)];
                    Vx[v] = Vx[v] - (dtr * d) / dx;
                }
                if (tx < nVy[0] - 2 && ty < nVy[1] - 2 && tz < nVy[2] - 2) {
                    int64_t v = OIDX(tx + 1, ty + 1, tz + 1, nVy);
                    REAL d = P[OIDX(tx + 1, ty + 1, tz + 1, n)] - P[OIDX(tx + 1, ty, tz + 1, n)];
                    Vy[v] = Vy[v] - (dtr * d) / dy;
                }
                if (tx < nVz[0] - 2 && ty < nVz[1] - 2 && tz < nVz[2] - 2) {
                    int64_t v = OIDX(tx + 1, ty + 1, tz + 1, nVz);
                    REAL d = P[OIDX(tx + 1, ty + 1, tz + 1, n)] - P[OIDX(tx + 1, ty + 1, tz, n)];
                    Vz[v] = Vz[v] - (dtr * d) / dz;
                }
            }
    return ORC_OK;
}

/* acoustic3D compute_P! (miniapps/acoustic3D.jl:18-21). */
int SFX(orc_acoustic3d_p)(REAL* P, const REAL* Vx, const REAL* Vy, const REAL* Vz, const int64_t* n, REAL dt,
                          REAL k, REAL dx, REAL dy, REAL dz) {
    int64_t nx = n[0], ny = n[1], nz = n[2];
    int64_t nVx[3] = {nx + 1, ny, nz}, nVy[3] = {nx, ny + 1, nz}, nVz[3] = {nx, ny, nz + 1};
    REAL dtk = dt * k;
#pragma omp parallel for schedule(static)
    for (int64_t iz = 0; iz < nz; iz++)
        for (int64_t iy = 0; iy < ny; iy++)
            for (int64_t ix = 0; ix < nx; ix++) {
                REAL ax = Vx[OIDX(ix + 1, iy, iz, nVx)] - Vx[OIDX(ix, iy, iz, nVx)];
                REAL ay = Vy[OIDX(ix, iy + 1, iz, nVy)] - Vy[OIDX(ix, iy, iz, nVy)];
                REAL az = Vz[OIDX(ix, iy, iz + 1, nVz)] - Vz[OIDX(ix, iy, iz, nVz)];
                int64_t p = OIDX(ix, iy, iz, n);
                P[p] = P[p] - dtk * ((ax / dx + ay / dy) + az / dz);
            }
    return ORC_OK;
}

/* ------------------------------------------------------------------------------------- */
/* Stokes2D miniapp kernels (miniapps/Stokes2D.jl:11-55). nx, ny: cell counts. Arrays:    */
/* Pt, dtPt, divV, txx, tyy, Mus, Rog (nx,ny); Vx (nx+1,ny); Vy (nx,ny+1); txy (nx-1,ny-1);*/
/* Rx, dVxdt, dtVx (nx-1,ny-2); Ry, dVydt, dtVy (nx-2,ny-1). A[ix + n0*iy].               */
/* ------------------------------------------------------------------------------------- */
#define I2(a, b, n0) ((int64_t)(a) + (int64_t)(n0) * (int64_t)(b))

/* compute_timesteps! (Stokes2D.jl:11-16): grid (nx, ny). */
int SFX(orc_stokes2d_timesteps)(REAL* dtVx, REAL* dtVy, REAL* dtPt, const REAL* Mus, int64_t nx, int64_t ny, REAL Vsc,
                                REAL Ptsc, REAL min_dxy2, int64_t max_nxy) {
    const REAL c41 = (REAL)4.1, h = (REAL)0.5, mn = (REAL)max_nxy;
#pragma omp parallel for schedule(static)
    for (int64_t ty = 0; ty < ny; ty++)
        for (int64_t tx = 0; tx < nx; tx++) {
            if (tx < nx - 1 && ty < ny - 2) {
                REAL av = (Mus[I2(tx, ty + 1, nx)] + Mus[I2(tx + 1, ty + 1, nx)]) * h;
                dtVx[I2(tx, ty, nx - 1)] = ((Vsc * min_dxy2) / av) / c41;
            }
            if (tx < nx - 2 && ty < ny - 1) {
                REAL av = (Mus[I2(tx + 1, ty, nx)] + Mus[I2(tx + 1, ty + 1, nx)]) * h;
                dtVy[I2(tx, ty, nx - 2)] = ((Vsc * min_dxy2) / av) / c41;
            }
            dtPt[I2(tx, ty, nx)] = ((Ptsc * c41) * Mus[I2(tx, ty, nx)]) / mn;
        }
    return ORC_OK;
}

/* compute_P! (Stokes2D.jl:18-22): grid (nx+1, ny+1); statements masked by @all(divV), @all(Pt). */
int SFX(orc_stokes2d_P)(REAL* divV, REAL* Pt, const REAL* Vx, const REAL* Vy, const REAL* dtPt, int64_t nx, int64_t ny,
                        REAL dx, REAL dy) {
#pragma omp parallel for schedule(static)
    for (int64_t ty = 0; ty < ny; ty++)
        for (int64_t tx = 0; tx < nx; tx++) {
            int64_t c = I2(tx, ty, nx);
            divV[c] = (Vx[I2(tx + 1, ty, nx + 1)] - Vx[I2(tx, ty, nx + 1)]) / dx +
                      (Vy[I2(tx, ty + 1, nx)] - Vy[I2(tx, ty, nx)]) / dy;
            Pt[c] = Pt[c] - dtPt[c] * divV[c];
        }
    return ORC_OK;
}

/* compute_τ! (Stokes2D.jl:24-29): grid (nx+1, ny+1). */
int SFX(orc_stokes2d_tau)(const REAL* divV, REAL* txx, REAL* tyy, REAL* txy, const REAL* Vx, const REAL* Vy,
                          const REAL* Mus, int64_t nx, int64_t ny, REAL dx, REAL dy) {
    const REAL two = (REAL)2.0, third = (REAL)1.0 / (REAL)3.0, h = (REAL)0.5, q = (REAL)0.25;
#pragma omp parallel for schedule(static)
    for (int64_t ty = 0; ty < ny; ty++)
        for (int64_t tx = 0; tx < nx; tx++) {
            int64_t c = I2(tx, ty, nx);
            REAL m2 = two * Mus[c];
            txx[c] = m2 * ((Vx[I2(tx + 1, ty, nx + 1)] - Vx[I2(tx, ty, nx + 1)]) / dx - third * divV[c]);
            tyy[c] = m2 * ((Vy[I2(tx, ty + 1, nx)] - Vy[I2(tx, ty, nx)]) / dy - third * divV[c]);
            if (tx < nx - 1 && ty < ny - 1) {
                REAL av = (((Mus[I2(tx, ty, nx)] + Mus[I2(tx + 1, ty, nx)]) + Mus[I2(tx, ty + 1, nx)]) +
                           Mus[I2(tx + 1, ty + 1, nx)]) * q;
                REAL dyVx = Vx[I2(tx + 1, ty + 1, nx + 1)] - Vx[I2(tx + 1, ty, nx + 1)];
                REAL dxVy = Vy[I2(tx + 1, ty + 1, nx)] - Vy[I2(tx, ty + 1, nx)];
                txy[I2(tx, ty, nx - 1)] = (two * av) * (h * (dyVx / dy + dxVy / dx));
            }
        }
    return ORC_OK;
}

/* compute_dV! (Stokes2D.jl:31-37): grid (nx, ny). */
int SFX(orc_stokes2d_dV)(REAL* Rx, REAL* Ry, REAL* dVxdt, REAL* dVydt, const REAL* Pt, const REAL* Rog, const REAL* txx,
                         const REAL* tyy, const REAL* txy, int64_t nx, int64_t ny, REAL dampX, REAL dampY, REAL dx,
                         REAL dy) {
    const REAL h = (REAL)0.5;
#pragma omp parallel for schedule(static)
    for (int64_t ty = 0; ty < ny; ty++)
        for (int64_t tx = 0; tx < nx; tx++) {
            if (tx < nx - 1 && ty < ny - 2) {
                int64_t r = I2(tx, ty, nx - 1);
                REAL a = txx[I2(tx + 1, ty + 1, nx)] - txx[I2(tx, ty + 1, nx)];
                REAL b = txy[I2(tx, ty + 1, nx - 1)] - txy[I2(tx, ty, nx - 1)];
                REAL c = Pt[I2(tx + 1, ty + 1, nx)] - Pt[I2(tx, ty + 1, nx)];
                Rx[r] = (a / dx + b / dy) - c / dx;
                dVxdt[r] = dampX * dVxdt[r] + Rx[r];
            }
            if (tx < nx - 2 && ty < ny - 1) {
                int64_t r = I2(tx, ty, nx - 2);
                REAL a = tyy[I2(tx + 1, ty + 1, nx)] - tyy[I2(tx + 1, ty, nx)];
                REAL b = txy[I2(tx + 1, ty, nx - 1)] - txy[I2(tx, ty, nx - 1)];
                REAL c = Pt[I2(tx + 1, ty + 1, nx)] - Pt[I2(tx + 1, ty, nx)];
                REAL g = (Rog[I2(tx + 1, ty, nx)] + Rog[I2(tx + 1, ty + 1, nx)]) * h;
                Ry[r] = ((a / dy + b / dx) - c / dy) + g;
                dVydt[r] = dampY * dVydt[r] + Ry[r];
            }
        }
    return ORC_OK;
}

/* compute_V! (Stokes2D.jl:39-43): grid (nx+1, ny+1); @inn(Vx), @inn(Vy). */
int SFX(orc_stokes2d_V)(REAL* Vx, REAL* Vy, const REAL* dVxdt, const REAL* dVydt, const REAL* dtVx, const REAL* dtVy,
                        int64_t nx, int64_t ny) {
#pragma omp parallel for schedule(static)
    for (int64_t ty = 0; ty < ny; ty++)
        for (int64_t tx = 0; tx < nx; tx++) {
            if (tx < nx - 1 && ty < ny - 2) {
                int64_t v = I2(tx + 1, ty + 1, nx + 1), r = I2(tx, ty, nx - 1);
                Vx[v] = Vx[v] + dtVx[r] * dVxdt[r];
            }
            if (tx < nx - 2 && ty < ny - 1) {
                int64_t v = I2(tx + 1, ty + 1, nx), r = I2(tx, ty, nx - 2);
                Vy[v] = Vy[v] + dtVy[r] * dVydt[r];
            }
        }
    return ORC_OK;
}

/* bc_x! / bc_y! (Stokes2D.jl:45-55): copy the first inner line onto the boundary line. */
int SFX(orc_bc_x2d)(REAL* A, int64_t n0, int64_t n1) {
    for (int64_t iy = 0; iy < n1; iy++) {
        A[I2(0, iy, n0)] = A[I2(1, iy, n0)];
        A[I2(n0 - 1, iy, n0)] = A[I2(n0 - 2, iy, n0)];
    }
    return ORC_OK;
}
int SFX(orc_bc_y2d)(REAL* A, int64_t n0, int64_t n1) {
    for (int64_t ix = 0; ix < n0; ix++) {
        A[I2(ix, 0, n0)] = A[I2(ix, 1, n0)];
        A[I2(ix, n1 - 1, n0)] = A[I2(ix, n1 - 2, n0)];
    }
    return ORC_OK;
}
/* ------------------------------------------------------------------------------------- */
/* Stokes2D, accelerated pseudo-transient (APT) iteration with pseudo-time steps from the   */
/* local viscosity maximum. No counterpart kernel in the reference: its Stokes2D miniapp's  */
/* damped iteration (above) diverges at viscosity contrasts of 1e-3; this scheme keeps the  */
/* miniapp's staggered arrays and statements (∇V, P, τ, R, V, free-slip copies) but relaxes */
/* the stresses in pseudo-time, with every local pseudo-time step taken from @maxloc(Mus)   */
/* (the reference's own idiom for heterogeneous coefficients, miniapps/HydroMech2D.jl:27):  */
/*   Musτ = Mus; @inn(Musτ) = @maxloc(Mus)                                                 */
/*   dτρ = ((Vpdτ*max_lxy)/Re)/Musτ, Gdτ = ((Vpdτ*Vpdτ)/dτρ)/(r+2)        (cells)           */
/*   kP = r*Gdτ, aτ = 1/(Gdτ/Mus + 1), bτ = (2*Gdτ)*aτ                    (cells)           */
/*   corner: Gc = min of the four cells' Gdτ, μc = @av(Mus), aτc, bτc as above             */
/*   face pseudo-steps: dτVx, dτVy = min of the two cells' dτρ                              */
/* One iteration (all differences times 1/dx, 1/dy):                                       */
/*   ∇V = dVx*_dx + dVy*_dy;  P = P - kP*∇V                                                 */
/*   τxx = aτ*τxx + bτ*(dVx*_dx - ∇V*(1/3));  τyy likewise;  τxy = aτc*τxy + bτc*εxy        */
/*   Rx = (dτxx*_dx + dτxy*_dy) - dP*_dx;  Ry = ((dτyy*_dy + dτxy*_dx) - dP*_dy) + @av_yi(Rog)*/
/*   V = V + dτV*R;  bc_y!(Vx), bc_x!(Vy)                                                   */
/* The coefficients are computed in FP64 from the field's own Mus values (FP32 arrays hold  */
/* their FP64 values rounded).                                                              */
/* ------------------------------------------------------------------------------------- */
#define I2(a, b, n0) ((int64_t)(a) + (int64_t)(n0) * (int64_t)(b))
#ifndef ORC_APT_COEFFS_DEFINED
#define ORC_APT_COEFFS_DEFINED
/* Coefficient arrays from Mus (FP64 only). Must: (nx, ny); kP, aT, bT: (nx, ny);
 * aTc, bTc: (nx-1, ny-1); dtVx: (nx-1, ny-2); dtVy: (nx-2, ny-1). */
int orc_stokes2d_apt_coeffs(double* Must, double* kP, double* aT, double* bT, double* aTc, double* bTc, double* dtVx,
                            double* dtVy, const double* Mus, int64_t nx, int64_t ny, double Vpdt, double Re, double r,
                            double max_lxy) {
    if (nx < 3 || ny < 3) return ORC_ERR_SHAPE;
    const int64_t n = nx * ny;
    double* G = (double*)malloc((size_t)n * sizeof(double));
    double* R = (double*)malloc((size_t)n * sizeof(double));
    if (!G || !R) {
        free(G);
        free(R);
        return ORC_ERR_ARG;
    }
    memcpy(Must, Mus, (size_t)n * sizeof(double));
    for (int64_t iy = 1; iy < ny - 1; iy++)
        for (int64_t ix = 1; ix < nx - 1; ix++) {
            /* @maxloc (src/FiniteDifferences.jl:189-190): max(max(max(W, E), C), max(S, N)) */
            double a = jl_max_f64(Mus[I2(ix - 1, iy, nx)], Mus[I2(ix + 1, iy, nx)]);
            a = jl_max_f64(a, Mus[I2(ix, iy, nx)]);
            Must[I2(ix, iy, nx)] = jl_max_f64(a, jl_max_f64(Mus[I2(ix, iy - 1, nx)], Mus[I2(ix, iy + 1, nx)]));
        }
    const double c0 = (Vpdt * max_lxy) / Re, v2 = Vpdt * Vpdt, rp2 = r + 2.0;
    for (int64_t i = 0; i < n; i++) {
        R[i] = c0 / Must[i];
        G[i] = (v2 / R[i]) / rp2;
        kP[i] = r * G[i];
        aT[i] = 1.0 / (G[i] / Mus[i] + 1.0);
        bT[i] = (2.0 * G[i]) * aT[i];
    }
    for (int64_t iy = 0; iy < ny - 1; iy++)
        for (int64_t ix = 0; ix < nx - 1; ix++) {
            double g = jl_min_f64(jl_min_f64(G[I2(ix, iy, nx)], G[I2(ix + 1, iy, nx)]),
                                  jl_min_f64(G[I2(ix, iy + 1, nx)], G[I2(ix + 1, iy + 1, nx)]));
            double mc = (((Mus[I2(ix, iy, nx)] + Mus[I2(ix + 1, iy, nx)]) + Mus[I2(ix, iy + 1, nx)]) +
                         Mus[I2(ix + 1, iy + 1, nx)]) * 0.25;
            double a = 1.0 / (g / mc + 1.0);
            aTc[I2(ix, iy, nx - 1)] = a;
            bTc[I2(ix, iy, nx - 1)] = (2.0 * g) * a;
        }
    for (int64_t iy = 0; iy < ny - 2; iy++)
        for (int64_t ix = 0; ix < nx - 1; ix++)
            dtVx[I2(ix, iy, nx - 1)] = jl_min_f64(R[I2(ix, iy + 1, nx)], R[I2(ix + 1, iy + 1, nx)]);
    for (int64_t iy = 0; iy < ny - 1; iy++)
        for (int64_t ix = 0; ix < nx - 2; ix++)
            dtVy[I2(ix, iy, nx - 2)] = jl_min_f64(R[I2(ix + 1, iy, nx)], R[I2(ix + 1, iy + 1, nx)]);
    free(G);
    free(R);
    return ORC_OK;
}

/* The FP64 residual of a state (Vx, Vy, Pt) with the stresses at their pseudo-time steady
 * state, τ = 2μ(ε̇ - ∇V/3) (μ = Mus at cells, @av(Mus) at corners): Rx (nx-1, ny-2),
 * Ry (nx-2, ny-1), divV (nx, ny); txx, tyy, txy receive those stresses. */
int orc_stokes2d_apt_residual(double* Rx, double* Ry, double* divV, double* txx, double* tyy, double* txy,
                              const double* Vx, const double* Vy, const double* Pt, const double* Mus,
                              const double* Rog, int64_t nx, int64_t ny, double _dx, double _dy) {
    const double third = 1.0 / 3.0;
    for (int64_t iy = 0; iy < ny; iy++)
        for (int64_t ix = 0; ix < nx; ix++) {
            int64_t c = I2(ix, iy, nx);
            double dvx = Vx[I2(ix + 1, iy, nx + 1)] - Vx[I2(ix, iy, nx + 1)];
            double dvy = Vy[I2(ix, iy + 1, nx)] - Vy[I2(ix, iy, nx)];
            double d = dvx * _dx + dvy * _dy;
            double td = d * third;
            divV[c] = d;
            txx[c] = (2.0 * Mus[c]) * (dvx * _dx - td);
            tyy[c] = (2.0 * Mus[c]) * (dvy * _dy - td);
            if (ix < nx - 1 && iy < ny - 1) {
                double mc = (((Mus[I2(ix, iy, nx)] + Mus[I2(ix + 1, iy, nx)]) + Mus[I2(ix, iy + 1, nx)]) +
                             Mus[I2(ix + 1, iy + 1, nx)]) * 0.25;
                double e = 0.5 * ((Vx[I2(ix + 1, iy + 1, nx + 1)] - Vx[I2(ix + 1, iy, nx + 1)]) * _dy +
                                  (Vy[I2(ix + 1, iy + 1, nx)] - Vy[I2(ix, iy + 1, nx)]) * _dx);
                txy[I2(ix, iy, nx - 1)] = (2.0 * mc) * e;
            }
        }
    for (int64_t iy = 0; iy < ny - 2; iy++)
        for (int64_t ix = 0; ix < nx - 1; ix++)
            Rx[I2(ix, iy, nx - 1)] = ((txx[I2(ix + 1, iy + 1, nx)] - txx[I2(ix, iy + 1, nx)]) * _dx +
                                      (txy[I2(ix, iy + 1, nx - 1)] - txy[I2(ix, iy, nx - 1)]) * _dy) -
                                     (Pt[I2(ix + 1, iy + 1, nx)] - Pt[I2(ix, iy + 1, nx)]) * _dx;
    for (int64_t iy = 0; iy < ny - 1; iy++)
        for (int64_t ix = 0; ix < nx - 2; ix++)
            Ry[I2(ix, iy, nx - 2)] = (((tyy[I2(ix + 1, iy + 1, nx)] - tyy[I2(ix + 1, iy, nx)]) * _dy +
                                       (txy[I2(ix + 1, iy, nx - 1)] - txy[I2(ix, iy, nx - 1)]) * _dx) -
                                      (Pt[I2(ix + 1, iy + 1, nx)] - Pt[I2(ix + 1, iy, nx)]) * _dy) +
                                     (Rog[I2(ix + 1, iy, nx)] + Rog[I2(ix + 1, iy + 1, nx)]) * 0.5;
    return ORC_OK;
}
#endif

/* One APT iteration in place (cells and corners, then faces and the free-slip copies). */
int SFX(orc_stokes2d_apt_step)(REAL* Vx, REAL* Vy, REAL* Pt, REAL* txx, REAL* tyy, REAL* txy, REAL* divV, REAL* Rx,
                               REAL* Ry, const REAL* kP, const REAL* aT, const REAL* bT, const REAL* aTc,
                               const REAL* bTc, const REAL* dtVx, const REAL* dtVy, const REAL* Rog, int64_t nx,
                               int64_t ny, REAL _dx, REAL _dy) {
    const REAL third = (REAL)(1.0 / 3.0), h = (REAL)0.5;
#pragma omp parallel for schedule(static)
    for (int64_t iy = 0; iy < ny; iy++)
        for (int64_t ix = 0; ix < nx; ix++) {
            int64_t c = I2(ix, iy, nx);
            REAL dvx = Vx[I2(ix + 1, iy, nx + 1)] - Vx[I2(ix, iy, nx + 1)];
            REAL dvy = Vy[I2(ix, iy + 1, nx)] - Vy[I2(ix, iy, nx)];
            REAL d = dvx * _dx + dvy * _dy;
            REAL td = d * third;
            divV[c] = d;
            Pt[c] = Pt[c] - kP[c] * d;
            txx[c] = aT[c] * txx[c] + bT[c] * (dvx * _dx - td);
            tyy[c] = aT[c] * tyy[c] + bT[c] * (dvy * _dy - td);
            if (ix < nx - 1 && iy < ny - 1) {
                int64_t k = I2(ix, iy, nx - 1);
                REAL e = h * ((Vx[I2(ix + 1, iy + 1, nx + 1)] - Vx[I2(ix + 1, iy, nx + 1)]) * _dy +
                              (Vy[I2(ix + 1, iy + 1, nx)] - Vy[I2(ix, iy + 1, nx)]) * _dx);
                txy[k] = aTc[k] * txy[k] + bTc[k] * e;
            }
        }
#pragma omp parallel for schedule(static)
    for (int64_t iy = 0; iy < ny - 1; iy++)
        for (int64_t ix = 0; ix < nx - 1; ix++) {
            if (iy < ny - 2) {
                int64_t k = I2(ix, iy, nx - 1);
                REAL R = ((txx[I2(ix + 1, iy + 1, nx)] - txx[I2(ix, iy + 1, nx)]) * _dx +
                          (txy[I2(ix, iy + 1, nx - 1)] - txy[I2(ix, iy, nx - 1)]) * _dy) -
                         (Pt[I2(ix + 1, iy + 1, nx)] - Pt[I2(ix, iy + 1, nx)]) * _dx;
                Rx[k] = R;
                Vx[I2(ix + 1, iy + 1, nx + 1)] = Vx[I2(ix + 1, iy + 1, nx + 1)] + dtVx[k] * R;
            }
            if (ix < nx - 2) {
                int64_t k = I2(ix, iy, nx - 2);
                REAL R = (((tyy[I2(ix + 1, iy + 1, nx)] - tyy[I2(ix + 1, iy, nx)]) * _dy +
                           (txy[I2(ix + 1, iy, nx - 1)] - txy[I2(ix, iy, nx - 1)]) * _dx) -
                          (Pt[I2(ix + 1, iy + 1, nx)] - Pt[I2(ix + 1, iy, nx)]) * _dy) +
                         (Rog[I2(ix + 1, iy, nx)] + Rog[I2(ix + 1, iy + 1, nx)]) * h;
                Ry[k] = R;
                Vy[I2(ix + 1, iy + 1, nx)] = Vy[I2(ix + 1, iy + 1, nx)] + dtVy[k] * R;
            }
        }
    SFX(orc_bc_y2d)(Vx, nx + 1, ny);
    SFX(orc_bc_x2d)(Vy, nx, ny + 1);
    return ORC_OK;
}

#undef I2

#undef OIDX

/* ------------------------------------------------------------------------------------- */
/* Stokes3D miniapp kernels (miniapps/Stokes3D.jl:11-68). Arrays column-major; nx, ny, nz = */
/* size(Pt). Grid = max extents of each kernel's array arguments; one mask per statement.   */
/* ------------------------------------------------------------------------------------- */
#define I3(a, b, c, n0, n1) ((int64_t)(a) + (int64_t)(n0) * ((int64_t)(b) + (int64_t)(n1) * (int64_t)(c)))

/* compute_timesteps! (Stokes3D.jl:11-17): grid (nx, ny, nz). */
int SFX(orc_stokes3d_timesteps)(REAL* dtVx, REAL* dtVy, REAL* dtVz, REAL* dtPt, const REAL* M, int64_t nx, int64_t ny,
                                int64_t nz, REAL Vsc, REAL Ptsc, REAL min_dxyz2, int64_t max_nxyz) {
    const REAL c61 = (REAL)6.1, h = (REAL)0.5, mn = (REAL)max_nxyz;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                if (x < nx - 1 && y < ny - 2 && z < nz - 2) {
                    REAL av = (M[I3(x, y + 1, z + 1, nx, ny)] + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * h;
                    dtVx[I3(x, y, z, nx - 1, ny - 2)] = ((Vsc * min_dxyz2) / av) / c61;
                }
                if (x < nx - 2 && y < ny - 1 && z < nz - 2) {
                    REAL av = (M[I3(x + 1, y, z + 1, nx, ny)] + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * h;
                    dtVy[I3(x, y, z, nx - 2, ny - 1)] = ((Vsc * min_dxyz2) / av) / c61;
                }
                if (x < nx - 2 && y < ny - 2 && z < nz - 1) {
                    REAL av = (M[I3(x + 1, y + 1, z, nx, ny)] + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * h;
                    dtVz[I3(x, y, z, nx - 2, ny - 2)] = ((Vsc * min_dxyz2) / av) / c61;
                }
                dtPt[I3(x, y, z, nx, ny)] = ((Ptsc * c61) * M[I3(x, y, z, nx, ny)]) / mn;
            }
    return ORC_OK;
}

/* compute_P! (Stokes3D.jl:19-23): grid (nx+1, ny+1, nz+1); statements masked by @all(∇V), @all(Pt). */
int SFX(orc_stokes3d_P)(REAL* divV, REAL* Pt, const REAL* Vx, const REAL* Vy, const REAL* Vz, const REAL* dtPt,
                        int64_t nx, int64_t ny, int64_t nz, REAL dx, REAL dy, REAL dz) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                int64_t c = I3(x, y, z, nx, ny);
                divV[c] = ((Vx[I3(x + 1, y, z, nx + 1, ny)] - Vx[I3(x, y, z, nx + 1, ny)]) / dx +
                           (Vy[I3(x, y + 1, z, nx, ny + 1)] - Vy[I3(x, y, z, nx, ny + 1)]) / dy) +
                          (Vz[I3(x, y, z + 1, nx, ny)] - Vz[I3(x, y, z, nx, ny)]) / dz;
                Pt[c] = Pt[c] - dtPt[c] * divV[c];
            }
    return ORC_OK;
}

/* compute_τ! (Stokes3D.jl:25-33): grid (nx+1, ny+1, nz+1). */
int SFX(orc_stokes3d_tau)(const REAL* divV, REAL* txx, REAL* tyy, REAL* tzz, REAL* txy, REAL* txz, REAL* tyz,
                          const REAL* Vx, const REAL* Vy, const REAL* Vz, const REAL* M, int64_t nx, int64_t ny,
                          int64_t nz, REAL dx, REAL dy, REAL dz) {
    const REAL two = (REAL)2.0, third = (REAL)1.0 / (REAL)3.0, h = (REAL)0.5, q = (REAL)0.25;
    const int64_t X1 = nx + 1, Y1 = ny + 1;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                if (y < ny - 2 && z < nz - 2) {
                    int64_t c = I3(x, y + 1, z + 1, nx, ny);
                    REAL d = (Vx[I3(x + 1, y + 1, z + 1, X1, ny)] - Vx[I3(x, y + 1, z + 1, X1, ny)]) / dx;
                    txx[I3(x, y, z, nx, ny - 2)] = (two * M[c]) * (d - third * divV[c]);
                }
                if (x < nx - 2 && z < nz - 2) {
                    int64_t c = I3(x + 1, y, z + 1, nx, ny);
                    REAL d = (Vy[I3(x + 1, y + 1, z + 1, nx, Y1)] - Vy[I3(x + 1, y, z + 1, nx, Y1)]) / dy;
                    tyy[I3(x, y, z, nx - 2, ny)] = (two * M[c]) * (d - third * divV[c]);
                }
                if (x < nx - 2 && y < ny - 2) {
                    int64_t c = I3(x + 1, y + 1, z, nx, ny);
                    REAL d = (Vz[I3(x + 1, y + 1, z + 1, nx, ny)] - Vz[I3(x + 1, y + 1, z, nx, ny)]) / dz;
                    tzz[I3(x, y, z, nx - 2, ny - 2)] = (two * M[c]) * (d - third * divV[c]);
                }
                if (x < nx - 1 && y < ny - 1 && z < nz - 2) {
                    REAL av = (((M[I3(x, y, z + 1, nx, ny)] + M[I3(x + 1, y, z + 1, nx, ny)]) +
                                M[I3(x, y + 1, z + 1, nx, ny)]) + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * q;
                    REAL a = Vx[I3(x + 1, y + 1, z + 1, X1, ny)] - Vx[I3(x + 1, y, z + 1, X1, ny)];
                    REAL b = Vy[I3(x + 1, y + 1, z + 1, nx, Y1)] - Vy[I3(x, y + 1, z + 1, nx, Y1)];
                    txy[I3(x, y, z, nx - 1, ny - 1)] = (two * av) * (h * (a / dy + b / dx));
                }
                if (x < nx - 1 && y < ny - 2 && z < nz - 1) {
                    REAL av = (((M[I3(x, y + 1, z, nx, ny)] + M[I3(x + 1, y + 1, z, nx, ny)]) +
                                M[I3(x, y + 1, z + 1, nx, ny)]) + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * q;
                    REAL a = Vx[I3(x + 1, y + 1, z + 1, X1, ny)] - Vx[I3(x + 1, y + 1, z, X1, ny)];
                    REAL b = Vz[I3(x + 1, y + 1, z + 1, nx, ny)] - Vz[I3(x, y + 1, z + 1, nx, ny)];
                    txz[I3(x, y, z, nx - 1, ny - 2)] = (two * av) * (h * (a / dz + b / dx));
                }
                if (x < nx - 2 && y < ny - 1 && z < nz - 1) {
                    REAL av = (((M[I3(x + 1, y, z, nx, ny)] + M[I3(x + 1, y + 1, z, nx, ny)]) +
                                M[I3(x + 1, y, z + 1, nx, ny)]) + M[I3(x + 1, y + 1, z + 1, nx, ny)]) * q;
                    REAL a = Vy[I3(x + 1, y + 1, z + 1, nx, Y1)] - Vy[I3(x + 1, y + 1, z, nx, Y1)];
                    REAL b = Vz[I3(x + 1, y + 1, z + 1, nx, ny)] - Vz[I3(x + 1, y, z + 1, nx, ny)];
                    tyz[I3(x, y, z, nx - 2, ny - 1)] = (two * av) * (h * (a / dz + b / dy));
                }
            }
    return ORC_OK;
}

/* compute_dV! (Stokes3D.jl:35-43): grid (nx, ny, nz). */
int SFX(orc_stokes3d_dV)(REAL* Rx, REAL* Ry, REAL* Rz, REAL* dVxdt, REAL* dVydt, REAL* dVzdt, const REAL* Pt,
                         const REAL* Rog, const REAL* txx, const REAL* tyy, const REAL* tzz, const REAL* txy,
                         const REAL* txz, const REAL* tyz, int64_t nx, int64_t ny, int64_t nz, REAL dampX, REAL dampY,
                         REAL dampZ, REAL dx, REAL dy, REAL dz) {
    const REAL h = (REAL)0.5;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                if (x < nx - 1 && y < ny - 2 && z < nz - 2) {
                    int64_t r = I3(x, y, z, nx - 1, ny - 2);
                    REAL a = txx[I3(x + 1, y, z, nx, ny - 2)] - txx[I3(x, y, z, nx, ny - 2)];
                    REAL b = txy[I3(x, y + 1, z, nx - 1, ny - 1)] - txy[I3(x, y, z, nx - 1, ny - 1)];
                    REAL c = txz[I3(x, y, z + 1, nx - 1, ny - 2)] - txz[I3(x, y, z, nx - 1, ny - 2)];
                    REAL p = Pt[I3(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3(x, y + 1, z + 1, nx, ny)];
                    Rx[r] = ((a / dx + b / dy) + c / dz) - p / dx;
                    dVxdt[r] = dampX * dVxdt[r] + Rx[r];
                }
                if (x < nx - 2 && y < ny - 1 && z < nz - 2) {
                    int64_t r = I3(x, y, z, nx - 2, ny - 1);
                    REAL a = tyy[I3(x, y + 1, z, nx - 2, ny)] - tyy[I3(x, y, z, nx - 2, ny)];
                    REAL b = txy[I3(x + 1, y, z, nx - 1, ny - 1)] - txy[I3(x, y, z, nx - 1, ny - 1)];
                    REAL c = tyz[I3(x, y, z + 1, nx - 2, ny - 1)] - tyz[I3(x, y, z, nx - 2, ny - 1)];
                    REAL p = Pt[I3(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3(x + 1, y, z + 1, nx, ny)];
                    Ry[r] = ((a / dy + b / dx) + c / dz) - p / dy;
                    dVydt[r] = dampY * dVydt[r] + Ry[r];
                }
                if (x < nx - 2 && y < ny - 2 && z < nz - 1) {
                    int64_t r = I3(x, y, z, nx - 2, ny - 2);
                    REAL a = tzz[I3(x, y, z + 1, nx - 2, ny - 2)] - tzz[I3(x, y, z, nx - 2, ny - 2)];
                    REAL b = txz[I3(x + 1, y, z, nx - 1, ny - 2)] - txz[I3(x, y, z, nx - 1, ny - 2)];
                    REAL c = tyz[I3(x, y + 1, z, nx - 2, ny - 1)] - tyz[I3(x, y, z, nx - 2, ny - 1)];
                    REAL p = Pt[I3(x + 1, y + 1, z + 1, nx, ny)] - Pt[I3(x + 1, y + 1, z, nx, ny)];
                    REAL g = (Rog[I3(x + 1, y + 1, z, nx, ny)] + Rog[I3(x + 1, y + 1, z + 1, nx, ny)]) * h;
                    Rz[r] = (((a / dz + b / dx) + c / dy) - p / dz) + g;
                    dVzdt[r] = dampZ * dVzdt[r] + Rz[r];
                }
            }
    return ORC_OK;
}

/* compute_V! (Stokes3D.jl:45-50): grid (nx+1, ny+1, nz+1); @inn(Vx), @inn(Vy), @inn(Vz). */
int SFX(orc_stokes3d_V)(REAL* Vx, REAL* Vy, REAL* Vz, const REAL* dVxdt, const REAL* dVydt, const REAL* dVzdt,
                        const REAL* dtVx, const REAL* dtVy, const REAL* dtVz, int64_t nx, int64_t ny, int64_t nz) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; z++)
        for (int64_t y = 0; y < ny; y++)
            for (int64_t x = 0; x < nx; x++) {
                if (x < nx - 1 && y < ny - 2 && z < nz - 2) {
                    int64_t v = I3(x + 1, y + 1, z + 1, nx + 1, ny), r = I3(x, y, z, nx - 1, ny - 2);
                    Vx[v] = Vx[v] + dtVx[r] * dVxdt[r];
                }
                if (x < nx - 2 && y < ny - 1 && z < nz - 2) {
                    int64_t v = I3(x + 1, y + 1, z + 1, nx, ny + 1), r = I3(x, y, z, nx - 2, ny - 1);
                    Vy[v] = Vy[v] + dtVy[r] * dVydt[r];
                }
                if (x < nx - 2 && y < ny - 2 && z < nz - 1) {
                    int64_t v = I3(x + 1, y + 1, z + 1, nx, ny), r = I3(x, y, z, nx - 2, ny - 2);
                    Vz[v] = Vz[v] + dtVz[r] * dVzdt[r];
                }
            }
    return ORC_OK;
}

/* bc_x! / bc_y! / bc_z! (Stokes3D.jl:52-68): copy the first inner plane onto the boundary plane. */
int SFX(orc_bc_x3d)(REAL* A, int64_t n0, int64_t n1, int64_t n2) {
    for (int64_t k = 0; k < n2; k++)
        for (int64_t j = 0; j < n1; j++) {
            A[I3(0, j, k, n0, n1)] = A[I3(1, j, k, n0, n1)];
            A[I3(n0 - 1, j, k, n0, n1)] = A[I3(n0 - 2, j, k, n0, n1)];
        }
    return ORC_OK;
}
int SFX(orc_bc_y3d)(REAL* A, int64_t n0, int64_t n1, int64_t n2) {
    for (int64_t k = 0; k < n2; k++)
        for (int64_t i = 0; i < n0; i++) {
            A[I3(i, 0, k, n0, n1)] = A[I3(i, 1, k, n0, n1)];
            A[I3(i, n1 - 1, k, n0, n1)] = A[I3(i, n1 - 2, k, n0, n1)];
        }
    return ORC_OK;
}
int SFX(orc_bc_z3d)(REAL* A, int64_t n0, int64_t n1, int64_t n2) {
    for (int64_t j = 0; j < n1; j++)
        for (int64_t i = 0; i < n0; i++) {
            A[I3(i, j, 0, n0, n1)] = A[I3(i, j, 1, n0, n1)];
            A[I3(i, j, n2 - 1, n0, n1)] = A[I3(i, j, n2 - 2, n0, n1)];
        }
    return ORC_OK;
}
#undef I3
