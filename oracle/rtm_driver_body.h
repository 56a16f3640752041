/*
 * Per-shot RTM driver loop (forward source run, backward source
 * reconstruction + receiver back-propagation + imaging), restating the
 * control flow of kernel.cu:791-933 with the wavefield operations supplied
 * as macros.  TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * The includer defines REAL, SFX(name), DRV_NAME(name) and the operation
 * macros K_EQUAL, K_ADD, K_HYB1, K_HYB2, K_HYB3, K_DELIVER, K_BKEQUAL,
 * K_BKADD_EFF, K_DELIVER_EFF, K_BKADD, K_BKHYB1, K_BKHYB2, K_REL.  rtm_oracle.c maps them onto
 * the restated loops of rtm_oracle_body.h; the reference build recipe in
 * this directory maps them onto the reference's own kernel bodies run on
 * the CPU, so both share this loop.
 *
 * Parameters are an or_params block (rtm_oracle.h).  Buffers are full grids
 * of NZ*NX values unless stated.
 */

/* Cells of the receivers: the reference's surface line (s_z, s_l + j*ds,
 * j < n) or an explicit list.  Returns the count. */
static int DRV_NAME(rec_cells)(const or_params *P, int *out)
{
    if (P->rec_cells) {
        for (int j = 0; j < P->nrec_list; ++j) out[j] = P->rec_cells[j];
        return P->nrec_list;
    }
    for (int j = 0; j < P->n; ++j) out[j] = P->s_z * P->NX + P->s_l + j * P->ds;
    return P->n;
}

/* Forward run of one shot (kernel.cu:798-821).  Returns the boundary rings
 * (caller-owned, NT slots) and the last two levels; when rec != NULL also
 * samples every level u_k (k = 0..NT-1, after the boundary blend) at the
 * receiver cells into rec[j*NT + k]. */
static int DRV_NAME(forward)(const or_params *P, const float *v, const float *r1,
                             const float *w, const float *c, const int *idx,
                             const float *wav, REAL *lf, REAL *rt, REAL *up, REAL *dw,
                             REAL *u0, REAL *u1, REAL *u2, REAL *b, REAL *rec)
{
    long nxz = (long)P->NZ * P->NX;
    int *cells = NULL, nr = 0;
    if (rec) {
        int cap = P->rec_cells ? P->nrec_list : P->n;
        cells = (int *)malloc(sizeof(int) * (cap > 0 ? cap : 1));
        if (!cells) return -1;
        nr = DRV_NAME(rec_cells)(P, cells);
    }
    for (long i = 0; i < nxz; ++i) { u0[i] = 0; u1[i] = 0; u2[i] = 0; b[i] = 0; }
    u1[(long)P->r_u * P->NX + P->r_x] = P->spike;
    K_EQUAL(lf, rt, up, dw, u0, u1);
    if (rec)
        for (int j = 0; j < nr; ++j) {
            rec[(long)j * P->NT + 0] = u0[cells[j]];
            rec[(long)j * P->NT + 1] = u1[cells[j]];
        }
    for (int k = 2; k < P->NT; ++k) {
        float wavelet = (k < P->NT2) ? wav[k - 1] : 0.0f;
        K_ADD(u2, u0, u1, wavelet);
        K_HYB1(u1, u0, u2, b);
        K_HYB2(u1, u0, u2, b);
        K_HYB3(u1, u0, u2, b, k);
        K_DELIVER(u1, u0, u2);
        if (rec)
            for (int j = 0; j < nr; ++j) rec[(long)j * P->NT + k] = u1[cells[j]];
    }
    free(cells);
    return 0;
}

/* Migration of one shot (kernel.cu:798-933): forward run, hand-off of the
 * last two levels, image/accumulator initialisation from the host arrays as
 * the reference leaves them (kernel.cu:859-885: the forward arrays on the
 * host still hold the initial state, zeros plus the start spike), then the
 * backward loop k = NT-3 .. 0.  seis is trace-major [ntrace][NT].  Outputs
 * rel1 (cross-correlation) and rel2 (source illumination), full grid. */
int DRV_NAME(migrate)(const or_params *P, const float *v, const float *r1, const float *w,
                      const float *c, const int *idx, const float *wav, const float *seis,
                      REAL *rel1, REAL *rel2)
{
    long nxz = (long)P->NZ * P->NX;
    int nz = P->NZ - 2 * P->N2, nx = P->NX - 2 * P->N2, M = P->M;
    long lfn = (long)M * nz * P->NT, upn = (long)M * nx * P->NT;
    REAL *lf = (REAL *)malloc(sizeof(REAL) * lfn), *rt = (REAL *)malloc(sizeof(REAL) * lfn);
    REAL *up = (REAL *)malloc(sizeof(REAL) * upn), *dw = (REAL *)malloc(sizeof(REAL) * upn);
    REAL *F0 = (REAL *)malloc(sizeof(REAL) * nxz), *F1 = (REAL *)malloc(sizeof(REAL) * nxz);
    REAL *F2 = (REAL *)malloc(sizeof(REAL) * nxz), *Fb = (REAL *)malloc(sizeof(REAL) * nxz);
    REAL *B0 = (REAL *)malloc(sizeof(REAL) * nxz), *B1 = (REAL *)malloc(sizeof(REAL) * nxz);
    REAL *B2 = (REAL *)malloc(sizeof(REAL) * nxz);
    REAL *FA = (REAL *)malloc(sizeof(REAL) * nxz), *BA = (REAL *)malloc(sizeof(REAL) * nxz);
    int ntr = P->rec_cells ? P->nrec_list : P->n;
    float *cs = (float *)malloc(sizeof(float) * (ntr > 0 ? ntr : 1));
    int *cells = (int *)malloc(sizeof(int) * (ntr > 0 ? ntr : 1));
    int rc = -1;
    if (!lf || !rt || !up || !dw || !F0 || !F1 || !F2 || !Fb || !B0 || !B1 || !B2 || !FA ||
        !BA || !cs || !cells)
        goto out;
    DRV_NAME(rec_cells)(P, cells);

    if (DRV_NAME(forward)(P, v, r1, w, c, idx, wav, lf, rt, up, dw, F0, F1, F2, Fb, NULL))
        goto out;
    /* Source side of the backward pass: B1 = u_{NT-2}, B0 = u_{NT-1}
     * (kernel.cu:822-825).  B2 starts at zero outside the interior. */
    for (long i = 0; i < nxz; ++i) { B1[i] = F0[i]; B0[i] = F1[i]; B2[i] = 0; }
    {
        /* kernel.cu:859-885 with the host forward arrays at their initial
         * state: h0 = 0 everywhere, h1 = spike at the source. */
        long src = (long)P->r_u * P->NX + P->r_x;
        for (long i = 0; i < nxz; ++i) {
            REAL h0 = 0, h1 = (i == src) ? (REAL)P->spike : (REAL)0;
            if (P->compen) {
                REAL bw2 = B0[i] + B1[i];
                REAL fw2 = h0 + h1;
                rel1[i] = fw2 * bw2 + h0 * B0[i];
                rel2[i] = B1[i] * B1[i] + B0[i] * B0[i];
                F2[i] = fw2; FA[i] = fw2; BA[i] = bw2;
            } else {
                rel1[i] = h1 * B1[i] + h0 * B0[i];
                rel2[i] = B1[i] * B1[i] + B0[i] * B0[i];
                F2[i] = 0; FA[i] = 0; BA[i] = 0;
            }
            Fb[i] = 0; F0[i] = 0; F1[i] = 0;
        }
    }
    for (int k = P->NT - 3; k >= 0; --k) {
        float wavelet = (k < P->NT2) ? wav[k + 1] : 0.0f;
        K_BKEQUAL(B1, k);
        K_BKADD_EFF(B2, B0, B1, wavelet);
        K_DELIVER_EFF(B1, B0, B2);
        for (int j = 0; j < ntr; ++j) cs[j] = seis[(long)j * P->NT + k + 1];
        K_BKADD(F2, F1, F0, cs);
        if (P->rec_cells)
            for (int j = 0; j < ntr; ++j)
                if (cs[j] != 0) F2[cells[j]] = cs[j];
        K_BKHYB1(F1, F0, F2, Fb);
        K_BKHYB2(F1, F0, F2, Fb);
        K_DELIVER(F1, F0, F2);
        K_REL(B2, F2, BA, FA, rel1, rel2);
    }
    rc = 0;
out:
    free(lf); free(rt); free(up); free(dw); free(F0); free(F1); free(F2); free(Fb);
    free(B0); free(B1); free(B2); free(FA); free(BA); free(cs); free(cells);
    return rc;
}

/* Forward modelling of one shot with receiver recording (new relative to the
 * reference, which reads recorded data from files): rec[j*NT + k] = u_k at
 * receiver j. */
int DRV_NAME(model)(const or_params *P, const float *v, const float *r1, const float *w,
                    const float *c, const int *idx, const float *wav, REAL *rec)
{
    long nxz = (long)P->NZ * P->NX;
    int nz = P->NZ - 2 * P->N2, nx = P->NX - 2 * P->N2, M = P->M;
    long lfn = (long)M * nz * P->NT, upn = (long)M * nx * P->NT;
    REAL *lf = (REAL *)malloc(sizeof(REAL) * lfn), *rt = (REAL *)malloc(sizeof(REAL) * lfn);
    REAL *up = (REAL *)malloc(sizeof(REAL) * upn), *dw = (REAL *)malloc(sizeof(REAL) * upn);
    REAL *F0 = (REAL *)malloc(sizeof(REAL) * nxz), *F1 = (REAL *)malloc(sizeof(REAL) * nxz);
    REAL *F2 = (REAL *)malloc(sizeof(REAL) * nxz), *Fb = (REAL *)malloc(sizeof(REAL) * nxz);
    int rc = -1;
    if (lf && rt && up && dw && F0 && F1 && F2 && Fb)
        rc = DRV_NAME(forward)(P, v, r1, w, c, idx, wav, lf, rt, up, dw, F0, F1, F2, Fb, rec);
    free(lf); free(rt); free(up); free(dw); free(F0); free(F1); free(F2); free(Fb);
    return rc;
}
