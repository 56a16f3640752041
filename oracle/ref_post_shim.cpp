/*
 * Post-stack routines of the reference used by the oracle's pin tests,
 * compiled from a caixh90/RTM_GPU checkout by build_ref.py into
 * oracle/_ref/libref_post.so.  TEST INFRASTRUCTURE ONLY.
 *   - DisToTimeAndTimeToDis1D.cpp (depth <-> time conversion of the image)
 *   - phase_correction_ricker_decon.cpp (constant phase rotation)
 * Both are included in place, unmodified, from the checkout's directory (a
 * translation unit of their own: LSMOrCon_rec_2D.cpp defines a macro `pi`).
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "DisToTimeAndTimeToDis1D.cpp"
#include "phase_correction_ricker_decon.cpp"

extern "C" {

/* D2T / T2D write their result to a file; these wrappers run them on a
 * scratch file and read the traces back into out (capacity cap floats). */
static int read_back(const char *path, float *out, long n)
{
    FILE *fh = fopen(path, "rb");
    if (!fh) return -1;
    long got = (long)fread(out, sizeof(float), n, fh);
    fclose(fh);
    return got == n ? 0 : -1;
}

int ref_d2t(const char *scratch, float *V, float *D, int Nx, int Nz, float dx, float dz, float dt,
            float *out, long cap)
{
    int nt = D2T(scratch, V, D, Nx, Nz, 0, Nx - 1, dx, dz, dt);
    if ((long)nt * Nx > cap || read_back(scratch, out, (long)nt * Nx)) return -1;
    return nt;
}

int ref_t2d(const char *scratch, float *V, float *D, int Nx, int Nt, int Nz_V, float dx, float dt,
            float dz, float *out, long cap)
{
    int nz = T2D(scratch, V, D, Nx, Nt, Nz_V, 0, Nx - 1, dx, dt, dz);
    if ((long)nz * Nx > cap || read_back(scratch, out, (long)nz * Nx)) return -1;
    return nz;
}

void ref_phase_correction(float *din, float *dout, int ntr, int nt, float angle)
{
    phase_correction(din, dout, ntr, nt, angle);
}

} /* extern "C" */
