/*
 * Wavefield kernels of the RTM hot path, restated as plain CPU loops.
 *
 * TEST INFRASTRUCTURE ONLY: this file is part of the CPU oracle. Nothing in
 * the product library includes it; tests, the smoke check and the CPU
 * baseline of bench.py are its only users.
 *
 * Included twice by rtm_oracle.c: once with REAL=float (the reference's own
 * precision; every mixed float/double expression of the reference is written
 * with the same literal types so that the same promotions happen) and once
 * with REAL=double (the FP64 oracle).  SFX(name) appends _f32 / _f64.
 *
 * Grid layout is the reference's: row-major [iz*NX + ix], iz = depth row,
 * ix = lateral column, NZ/NX include the N2-wide absorbing pad.
 */

/* ---- boundary-ring store (kernel.cu:18-45 Equal, :184-208 Hybrid3,
 *      :222-245 BKEqual).  Ring slot s holds, for the M cells just outside
 *      the interior on each of the four sides (corners excluded):
 *        lf[(s*nz + zi)*M + m] = u[(N2+zi)*NX + N2-1-m]
 *        rt[(s*nz + zi)*M + m] = u[(N2+zi)*NX + NX-N2+m]
 *        up[(s*M + m)*nx + xi] = u[(N2-1-m)*NX + N2+xi]
 *        dw[(s*M + m)*nx + xi] = u[(NZ-N2+m)*NX + N2+xi]                  */
static void SFX(ring_copy)(REAL *lf, REAL *rt, REAL *up, REAL *dw, REAL *u,
                           int NZ, int NX, int N2, int M, long slot, int restore)
{
    int nz = NZ - 2 * N2, nx = NX - 2 * N2;
    long oz = slot * (long)nz * M, ox = slot * (long)nx * M;
    for (int zi = 0; zi < nz; ++zi)
        for (int m = 0; m < M; ++m) {
            long ri = oz + (long)zi * M + m;
            long cl = (long)(N2 + zi) * NX + (N2 - 1 - m);
            long cr = (long)(N2 + zi) * NX + (NX - N2 + m);
            if (restore) { u[cl] = lf[ri]; u[cr] = rt[ri]; }
            else         { lf[ri] = u[cl]; rt[ri] = u[cr]; }
        }
    for (int m = 0; m < M; ++m)
        for (int xi = 0; xi < nx; ++xi) {
            long ri = ox + (long)m * nx + xi;
            long cu = (long)(N2 - 1 - m) * NX + (N2 + xi);
            long cd = (long)(NZ - N2 + m) * NX + (N2 + xi);
            if (restore) { u[cu] = up[ri]; u[cd] = dw[ri]; }
            else         { up[ri] = u[cu]; dw[ri] = u[cd]; }
        }
}

/* kernel.cu:18-45 (Equal): slots 0 and 1 from the first two time levels. */
void SFX(or_equal)(REAL *lf, REAL *rt, REAL *up, REAL *dw, REAL *u0, REAL *u1,
                   int NZ, int NX, int N2, int M)
{
    SFX(ring_copy)(lf, rt, up, dw, u0, NZ, NX, N2, M, 0, 0);
    SFX(ring_copy)(lf, rt, up, dw, u1, NZ, NX, N2, M, 1, 0);
}

/* kernel.cu:184-208 (Hybrid3): slot k from the blended new level. */
void SFX(or_ring_save)(REAL *lf, REAL *rt, REAL *up, REAL *dw, REAL *u2,
                       int NZ, int NX, int N2, int M, int k)
{
    SFX(ring_copy)(lf, rt, up, dw, u2, NZ, NX, N2, M, k, 0);
}

/* kernel.cu:222-245 (BKEqual): restores slot k+1 into u1. */
void SFX(or_bkequal)(REAL *lf, REAL *rt, REAL *up, REAL *dw, REAL *u1,
                     int NZ, int NX, int N2, int M, int k)
{
    SFX(ring_copy)(lf, rt, up, dw, u1, NZ, NX, N2, M, (long)k + 1, 1);
}

/* Even reflection about the first/last sample, as the stencils of
 * kernel.cu:65-68 do for out-of-range neighbours. */
static inline int SFX(mirror)(int i, int n)
{
    if (i < 0) return -i;
    if (i >= n) return 2 * n - 2 - i;
    return i;
}

/* Spatial part of the 2M-order operator at (z,x) (kernel.cu:59-72):
 *   w = (1+hzx2_1)*c[0]*u + sum_l c[l]*((u[z-l]+u[z+l])*hzx2_1 + u[x-l] + u[x+l])
 * The first product is formed in double and rounded once (the reference
 * writes it with the literal 1.0); the loop accumulates in REAL. */
static inline REAL SFX(lap)(const REAL *u1, const float *c, int nc_minus1,
                            int z, int x, int NZ, int NX, float hzx2_1)
{
    long i = (long)z * NX + x;
    REAL w1 = (1.0 + hzx2_1) * c[0] * u1[i];
    for (int l = 1; l <= nc_minus1; ++l) {
        int z1 = SFX(mirror)(z - l, NZ), z2 = SFX(mirror)(z + l, NZ);
        int x1 = SFX(mirror)(x - l, NX), x2 = SFX(mirror)(x + l, NX);
        w1 = w1 + c[l] * ((u1[(long)z1 * NX + x] + u1[(long)z2 * NX + x]) * hzx2_1
                          + u1[(long)z * NX + x1] + u1[(long)z * NX + x2]);
    }
    return w1;
}

/* Velocity-bin lookup of kernel.cu:55-57: the bin of a cell is
 * int((v-vmin)/dv + 0.5); its coefficients are c[Index[bin] .. Index[bin+1]-1]. */
static inline void SFX(bin_coefs)(float v, float vmin, float dv, const int *idx,
                                  int *top, int *cnt)
{
    int e = idx[(int)((v - vmin) / dv + 1.5)];
    int t = idx[(int)((v - vmin) / dv + 0.5)];
    *top = t;
    *cnt = e - t - 1;  /* loop runs l = 1 .. cnt */
}

/* kernel.cu:46-80 (Add, adaptive coefficients) and :82-114 (Add_Con, fixed
 * coefficients c[0..M]).  adaptive!=0 selects Add.  Full grid, source added
 * at (r_u, r_x) after the update. */
void SFX(or_add)(const float *v, REAL *u2, const REAL *u0, const REAL *u1,
                 const float *c, const int *idx, int adaptive, float tao2, float h2,
                 float vmin, float dv, int M, int NZ, int NX, int r_u, int r_x,
                 float wavelet, float hzx2_1)
{
#pragma omp parallel for schedule(static)
    for (int z = 0; z < NZ; ++z)
        for (int x = 0; x < NX; ++x) {
            long i = (long)z * NX + x;
            REAL w1;
            if (adaptive) {
                int top, cnt;
                SFX(bin_coefs)(v[i], vmin, dv, idx, &top, &cnt);
                w1 = SFX(lap)(u1, c + top, cnt, z, x, NZ, NX, hzx2_1);
                u2[i] = 2 * u1[i] - u0[i] + (REAL)v[i] * v[i] * tao2 * h2 * w1;
            } else {
                w1 = SFX(lap)(u1, c, M, z, x, NZ, NX, hzx2_1);
                u2[i] = 2.0 * u1[i] - u0[i] + (REAL)v[i] * v[i] * tao2 * h2 * w1;
            }
            if (z == r_u && x == r_x) u2[i] += wavelet;
        }
}

/* kernel.cu:246-283 (BKAdd_EFF) and :286-320 (BKAdd_EFF_Con): the same
 * update restricted to the interior [N2,NZ-N2) x [N2,NX-N2). */
void SFX(or_bkadd_eff)(const float *v, REAL *u2, const REAL *u0, const REAL *u1,
                       const float *c, const int *idx, int adaptive, float tao2, float h2,
                       float vmin, float dv, int M, int N2, int NZ, int NX, int r_u,
                       int r_x, float wavelet, float hzx2_1)
{
#pragma omp parallel for schedule(static)
    for (int z = N2; z < NZ - N2; ++z)
        for (int x = N2; x < NX - N2; ++x) {
            long i = (long)z * NX + x;
            REAL w1;
            if (adaptive) {
                int top, cnt;
                SFX(bin_coefs)(v[i], vmin, dv, idx, &top, &cnt);
                w1 = SFX(lap)(u1, c + top, cnt, z, x, NZ, NX, hzx2_1);
            } else {
                w1 = SFX(lap)(u1, c, M, z, x, NZ, NX, hzx2_1);
            }
            u2[i] = 2.0 * u1[i] - u0[i] + (REAL)v[i] * v[i] * tao2 * h2 * w1;
            if (z == r_u && x == r_x) u2[i] += wavelet;
        }
}

/* kernel.cu:339-380 (BKAdd) and :381-418 (BKAdd_Con): receiver-side update
 * on the full grid.  On the line z=s_z, x=s_l+s*ds<=s_r, a non-zero datum
 * seis[s] replaces the update (Dirichlet injection). */
void SFX(or_bkadd)(const float *v, REAL *u2, const REAL *u1, const REAL *u0,
                   const float *c, const int *idx, int adaptive, const float *seis,
                   float tao2, float h2, float vmin, float dv, int M, int NZ, int NX,
                   int s_l, int s_r, int s_z, int ds, float hzx2_1)
{
#pragma omp parallel for schedule(static)
    for (int z = 0; z < NZ; ++z)
        for (int x = 0; x < NX; ++x) {
            long i = (long)z * NX + x;
            if (z == s_z && x >= s_l && x <= s_r && (x - s_l) % ds == 0 &&
                seis[(x - s_l) / ds] != 0) {
                u2[i] = seis[(x - s_l) / ds];
                continue;
            }
            REAL w1;
            if (adaptive) {
                int top, cnt;
                SFX(bin_coefs)(v[i], vmin, dv, idx, &top, &cnt);
                w1 = SFX(lap)(u1, c + top, cnt, z, x, NZ, NX, hzx2_1);
            } else {
                w1 = SFX(lap)(u1, c, M, z, x, NZ, NX, hzx2_1);
            }
            u2[i] = 2 * u1[i] - u0[i] + (REAL)v[i] * v[i] * tao2 * h2 * w1;
        }
}

/* Receiver-list form of the Dirichlet injection (extension of the line rule
 * above to arbitrary receiver cells, e.g. a vertical well): a non-zero datum
 * replaces the value at its cell.  Applied after or_bkadd with an empty line. */
void SFX(or_inject_list)(REAL *u2, const int *cell, const float *d, int n)
{
    for (int j = 0; j < n; ++j)
        if (d[j] != 0) u2[cell[j]] = d[j];
}

/* ---- hybrid absorbing boundary (kernel.cu:116-183 Hybrid1/Hybrid2 and the
 *      identical BKHybrid1/2 at :421-487).
 *
 * Every cell of the N2-wide pad gets a one-way value b, then is blended
 * u2 = (1-w[j])*u2 + w[j]*b.  With a = distance to the nearer of the top /
 * bottom edges and e = distance to the nearer of the left / right edges:
 *   e >= a+2 : one-way update across the top or bottom edge,
 *   a >= e+2 : one-way update across the left or right edge,
 *   otherwise: the 45-degree corner update with r_1.
 *   j = max(N2-z, N2-x, z-(NZ-N2)+1, x-(NX-N2)+1).
 * These index sets are exactly the union of the thread conditions of
 * Hybrid1/Hybrid2 (checked by enumeration in the tests).
 *
 * Side update, cell c, inward neighbour n (one cell towards the interior),
 * lateral step s along the edge:
 *   b = 1/(taoh*v_c+1) * ( taoh*v_c*(u2[n]-u0[n]+u0[c])
 *        - (-2u1[c]+u0[c]+u2[n]-2u1[n]+u0[n])
 *        + taoh2*vq*vq*(u2[n+s]-2u2[n]+u2[n-s]+u0[c+s]-2u0[c]+u0[c-s]) )
 * vq is the velocity the reference reads for the lateral term:
 *   top  : v[c];                bottom: v[(NZ-1-z)*NX + x]  (kernel.cu:132)
 *   left : v[x*NX + z];         right : v[(NX-1-x)*NX + z]  (kernel.cu:128,136)
 * (flat indices; quirk=0 uses v[c] on all four sides instead).
 * Corner update with the two inward neighbours p (along x), q (along z):
 *   b = 1/(2*r1[c]+1) * (u1[c] + r1[c]*(u2[p]+u2[q]))
 * u2 is read before any blending (Hybrid2 runs after Hybrid1 completes). */
void SFX(or_hybrid1)(const REAL *u1, const REAL *u0, const REAL *u2, REAL *b,
                     const float *v, const float *r1, int NZ, int NX, int N2,
                     float taoh, float taoh2, int quirk)
{
#pragma omp parallel for schedule(static)
    for (int z = 0; z < NZ; ++z)
        for (int x = 0; x < NX; ++x) {
            if (z >= N2 && z < NZ - N2 && x >= N2 && x < NX - N2) continue;
            long c = (long)z * NX + x;
            int a = z < NZ - 1 - z ? z : NZ - 1 - z;
            int e = x < NX - 1 - x ? x : NX - 1 - x;
            int dz = (z < NZ - 1 - z) ? 1 : -1;   /* inward along z */
            int dx = (x < NX - 1 - x) ? 1 : -1;   /* inward along x */
            if (e >= a + 2 || a >= e + 2) {
                long n, s;
                long q;
                if (e >= a + 2) {           /* top / bottom edge */
                    n = c + (long)dz * NX;
                    s = 1;
                    q = (dz > 0) ? c : (long)(NZ - 1 - z) * NX + x;
                } else {                    /* left / right edge */
                    n = c + dx;
                    s = NX;
                    q = (dx > 0) ? (long)x * NX + z : (long)(NX - 1 - x) * NX + z;
                }
                if (!quirk) q = c;
                b[c] = 1 / ((REAL)taoh * v[c] + 1) *
                       ((REAL)taoh * v[c] * (u2[n] - u0[n] + u0[c]) -
                        (-2 * u1[c] + u0[c] + u2[n] - 2 * u1[n] + u0[n]) +
                        (REAL)taoh2 * v[q] * v[q] *
                            (u2[n + s] - 2 * u2[n] + u2[n - s] + u0[c + s] - 2 * u0[c] + u0[c - s]));
            } else {
                long p = c + dx, q = c + (long)dz * NX;
                b[c] = 1 / (2 * (REAL)r1[c] + 1) * (u1[c] + (REAL)r1[c] * (u2[p] + u2[q]));
            }
        }
}

static inline int SFX(blend_j)(int z, int x, int NZ, int NX, int N2)
{
    int j = N2 - z;
    if (N2 - x > j) j = N2 - x;
    if (z - (NZ - N2) + 1 > j) j = z - (NZ - N2) + 1;
    if (x - (NX - N2) + 1 > j) j = x - (NX - N2) + 1;
    return j;
}

void SFX(or_hybrid2)(REAL *u2, const REAL *b, const float *w, int NZ, int NX, int N2)
{
#pragma omp parallel for schedule(static)
    for (int z = 0; z < NZ; ++z)
        for (int x = 0; x < NX; ++x) {
            if (z >= N2 && z < NZ - N2 && x >= N2 && x < NX - N2) continue;
            long c = (long)z * NX + x;
            int j = SFX(blend_j)(z, x, NZ, NX, N2);
            u2[c] = (1 - w[j]) * u2[c] + w[j] * b[c];
        }
}

/* kernel.cu:210-221 (Deliver): u0 <- u1, u1 <- u2 over the full grid;
 * kernel.cu:323-337 (Deliver_EFF): the same on the interior only. */
void SFX(or_deliver)(REAL *u1, REAL *u0, const REAL *u2, int NZ, int NX, int N2, int interior)
{
    int lo = interior ? N2 : 0;
#pragma omp parallel for schedule(static)
    for (int z = lo; z < NZ - lo; ++z)
        for (int x = lo; x < NX - lo; ++x) {
            long i = (long)z * NX + x;
            u0[i] = u1[i];
            u1[i] = u2[i];
        }
}

/* kernel.cu:489-517 (Rel_NonCompen / Rel_Compen) over the full grid, with
 * S the source wavefield and R the receiver wavefield at the same step:
 *   compen=0: rel1 += R*S;                       rel2 += S*S
 *   compen=1: Sacc += S; Racc += R; rel1 += Racc*Sacc; rel2 += S*S        */
void SFX(or_rel)(const REAL *S, const REAL *R, REAL *Sacc, REAL *Racc, REAL *rel1,
                 REAL *rel2, int NZ, int NX, int compen)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)NZ * NX; ++i) {
        if (compen) {
            Sacc[i] += S[i];
            Racc[i] += R[i];
            rel1[i] += Racc[i] * Sacc[i];
        } else {
            rel1[i] += R[i] * S[i];
        }
        rel2[i] += S[i] * S[i];
    }
}
