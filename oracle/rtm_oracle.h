/*
 * CPU oracle for the RTM hot path of caixh90/RTM_GPU (kernel.cu,
 * LSMOrCon_rec_2D.cpp, GPU_velocity_real.cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against; only tests, the smoke check and bench.py's CPU-baseline leg load
 * it.  The product library never links, loads or calls anything here.
 *
 * Parity pin: the FP32 path is compared bit for bit with the reference's own
 * kernel bodies and optimiser run on the CPU (see build_ref.py and the golden
 * fixtures generated from it under tests/golden/).
 */
#ifndef RTM_ORACLE_H
#define RTM_ORACLE_H

/* Scalar block shared by the driver loops.  All fields are 4-byte; the two
 * pointers at the end describe an optional explicit receiver list. */
typedef struct {
    int NZ, NX, N2, M;        /* padded grid, pad width, nfdmax (ring width)   */
    int NT, NT2;              /* time steps, wavelet cut-off step              */
    int adaptive;             /* 1: per-bin coefficients (iLSTE=0), 0: fixed  */
    int compen;               /* iCompen                                       */
    int quirk;                /* 1: reference velocity indexing in the ABC     */
    int r_u, r_x;             /* source cell (0-based padded)                  */
    int s_l, s_r, s_z, ds, n; /* receiver line (0-based padded), n traces      */
    int nrec_list;            /* length of rec_cells when used                 */
    int pad_;
    float tao2, h2, taoh, taoh2, vmin, dv, hzx2_1, spike;
    const int *rec_cells;     /* NULL: use the line                            */
} or_params;

#endif
