/*
 * msk_oracle.h -- CPU restatement of the reference's multislice hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load this library, and only as the reference
 * the GPU results are compared with (or as the timed CPU baseline); the
 * shipped library never calls it.
 *
 * Two arithmetic variants of the same method:
 *   *_f32  mirrors the reference's own float/double mix operation by
 *          operation (TemsimLibrary/autoslic.cpp, slicelib.cpp, cfpix.cpp);
 *          linked with the same CPU FFT as oracle/_ref it reproduces the
 *          reference build bit for bit, which pins this restatement.
 *   *_f64  the FP64 oracle: the same method (same atoms per slice, same
 *          spline table, same band-limit and aperture decisions) with every
 *          value carried in double and a double FFT.
 *
 * Grids are complex, interleaved (re, im), x-major: element (ix, iy) at
 * index iy + ix*ny, as in the reference's cfpix (cfpix.hpp:117,133).
 * Parity is pinned against oracle/_ref (the reference compiled here) through
 * tests/golden fixtures; the FFT and the free-space step follow the
 * definitions documented in fft_cpu.h and mo_defocus_* below.
 */
#ifndef MSK_ORACLE_H
#define MSK_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* param[] offsets read by autoslic::calculate (slicelib.hpp:142-240). */
enum {
    MO_pXCTILT = 9, MO_pYCTILT = 10, MO_pDEFOCUS = 11, MO_pENERGY = 16, MO_pOAPERT = 17,
    MO_pCAPERT = 21, MO_pDDF = 22, MO_pDELTAZ = 30, MO_pAX = 101, MO_pBY = 102,
    MO_pNX = 104, MO_pNY = 105, MO_pNWOBBLE = 111, MO_pTEMPER = 120, MO_pCAPERTMIN = 121,
    MO_NPARAM = 200
};

/* Status codes (the reference calls exit(0) in these cases). */
enum {
    MO_OK = 0,
    MO_EBADSIZE = -1,   /* nx, ny < 1 or ax, by < 0 (autoslic.cpp:258-262) */
    MO_EBOX = -2,       /* atom outside [0,ctblength]^2 x [0,ctblengthz] (autoslic.cpp:288-299) */
    MO_EZSORT = -3,     /* sorted z outside [0, ctblengthz] (autoslic.cpp:734-739) */
    MO_EZNUM = -4,      /* atomic number outside 1..103 (slicelib.cpp:2847-2851) */
    MO_ENOMEM = -5
};

/* slicelib.cpp physics (restated) */
double mo_wavelength(double kev);
double mo_sigma(double kev);
void mo_freqn(float *ko, float *ko2, float *xo, int nk, double ak);
double mo_bessi0(double x);
double mo_bessk0(double x);
double mo_vzatom(int Z, double r);
void mo_splinh(const double *x, const double *y, double *b, double *c, double *d, int n);
double mo_seval(const double *x, const double *y, const double *b, const double *c,
                const double *d, int n, double x0);
double mo_vzatomLUT(int Z, double rsq);
/* The spline table: knots[100] (r^2) and coefficients y,b,c,d[100] for Z. */
int mo_lut_table(int Z, double *knots, double *y, double *b, double *c, double *d);

/* Host preparation (bit-exact with the reference; built with -ffp-contract=off). */
void mo_sortByZ(float *x, float *y, float *z, float *occ, int *Znum, int natom);
void mo_rotate(float ctblength, double dxc, double dyc, double dzc, double angleZ,
               double angleY, int natom, float *x, float *y, float *z);
int mo_drop_outside(float ctblength, float ctblengthz, int natom, float *x, float *y,
                    float *z, float *occ, int *Znum);
/* Number of slice-steps calculate() runs for a box of depth zmax (autoslic.cpp:747-830). */
int mo_slice_count(float deltaz, float zmax);
/* Slice index (0-based) of every atom of a z-sorted list; returns the slice count. */
int mo_slice_assign(float deltaz, float zmax, int natom, const float *zsorted, int *slice_of_atom);

/* autoslic::calculate, coherent branch (lpartl = lbeams = lcross = 0, no wobble).
 * max_slices < 0 runs every slice.  Returns MO_OK or a negative status. */
int mo_calculate_f32(float *pix, const float *wave0, const float *param, int natom,
                     const int *Znum, const float *x, const float *y, const float *z,
                     const float *occ, float ctblength, float ctblengthz, int nmode,
                     int max_slices);
/* The same loop over slices [min_slice, max_slices) only -- earlier slices'
 * atoms are skipped and no transforms run for them.  For timing samples:
 * the wave it returns is not the physical one. */
int mo_calculate_sample_f32(float *pix, const float *wave0, const float *param, int natom,
                            const int *Znum, const float *x, const float *y, const float *z,
                            const float *occ, float ctblength, float ctblengthz, int nmode,
                            int min_slice, int max_slices);
int mo_calculate_f64(double *pix, const double *wave0, const float *param, int natom,
                     const int *Znum, const float *x, const float *y, const float *z,
                     const float *occ, float ctblength, float ctblengthz, int nmode,
                     int max_slices);

/* Free-space propagation of an exit wave to a detector plane and |psi|^2.
 * This build's definition of the missing XArray2DFFT::FresnelA call
 * (autosliccmd.cpp:1060,1087) and Abs2 (autosliccmd.cpp:1208):
 *   Psi = fft(psi)  (the cfpix fft convention, kernel exp(+2 pi i ...))
 *   chi(k) = pi*lambda*R*k^2 + (pi/2)*Cs3*lambda^3*k^4 + (pi/3)*Cs5*lambda^5*k^6
 *            + (pi/2)*lambda*astig*((kx^2-ky^2)*cos(2 th) + 2 kx ky sin(2 th))
 *   Psi *= exp(-i chi) where k^2 < k2maxo (or everywhere if k2maxo == 0), else 0
 *   psi' = ifft(Psi) / (nx*ny);   I = |psi'|^2
 * with R = defocus - ctblengthz/2 (autosliccmd.cpp:1060), k from freqn(),
 * chi evaluated in double and reduced modulo 2 pi before the sine/cosine.
 * lambda, cs3 and cs5 in Angstrom.  inten_out gets nx*ny floats (doubles). */
int mo_defocus_f32(const float *pix, int nx, int ny, float ax, float by, double wavlen,
                   double rprime, float k2maxo, double cs3, double cs5, double astig,
                   double astig_angle, float *inten_out);
int mo_defocus_f64(const double *pix, int nx, int ny, float ax, float by, double wavlen,
                   double rprime, float k2maxo, double cs3, double cs5, double astig,
                   double astig_angle, double *inten_out);

/* One orientation of MsctKirkland's per-angle worker (autosliccmd.cpp:711-748,
 * 936, 1051-1087, 1205-1224), FP32 mirror: rotate the specimen, drop atoms
 * outside the box, calculate() from a plane wave, then one intensity image
 * per defocus.  disp (optional): float[3][natom] added to the rotated
 * coordinates before the box rule (a frozen-phonon configuration).
 * images: ndef * nx*ny floats.  exitwave (optional): 2*nx*ny.
 * Returns the number of atoms kept, or a negative status. */
typedef struct {
    float ax;           /* field of view = ctblength, Angstrom */
    float ctblengthz;   /* box depth, Angstrom */
    int nx, ny;
    float v0;           /* keV */
    float deltaz;       /* slice thickness, Angstrom */
    float aobj;         /* objective aperture, rad (0 = none) */
    double cs3, cs5;    /* Angstrom */
    double dxc, dyc, dzc;  /* rotation centre shifts, Angstrom */
    int nmode;
    int max_slices;     /* < 0: all */
    int min_slice;      /* slices before it are skipped (cost samples only) */
} mo_series_params;

int mo_orientation_f32(const mo_series_params *sp, int natom, const int *Znum,
                       const float *x, const float *y, const float *z, const float *occ,
                       double angleZ, double angleY, const float *disp, int ndef,
                       const double *defocus,
                       float *images, float *exitwave);
int mo_orientation_f64(const mo_series_params *sp, int natom, const int *Znum,
                       const float *x, const float *y, const float *z, const float *occ,
                       double angleZ, double angleY, const float *disp, int ndef,
                       const double *defocus,
                       double *images, double *exitwave);

/* Many orientations on nthreads host threads (one orientation per thread at
 * a time, as MsctKirkland drives the reference, MultisliceT.cpp:403-448).
 * Atom arrays of unit u start at x + u*coord_stride (coord_stride 0: one
 * shared specimen; natom: per-unit displaced copies for frozen-phonon
 * configurations); the unit's angles are angZ[u], angY[u].
 * images: nunits * ndef * nx*ny.  Returns MO_OK or the first failure. */
int mo_orientations_f32(const mo_series_params *sp, int nunits, int nthreads, int natom,
                        long coord_stride, const int *Znum, const float *x, const float *y,
                        const float *z, const float *occ, const double *angZ,
                        const double *angY, int ndef, const double *defocus, float *images);

/* Per-slice projected potentials (FP64 sums) of one orientation, sliced as
 * calculate() slices it: v[mo_slice_count(deltaz, ctblengthz)][nx][ny].
 * Returns the atoms kept or a negative status. */
int mo_orientation_potential_f64(const mo_series_params *sp, int natom, const int *Znum,
                                 const float *x, const float *y, const float *z,
                                 const float *occ, double angleZ, double angleY, double *v);

/* Image plane of a detector (autosliccmd.cpp:1119-1143, this project's
 * definitions of the missing XArrayLibrary calls): rotation by theta about
 * (xc, yc), then a whole-pixel shift (sx, sy), in place on amp [nx][ny]. */
void mo_image_plane_f64(double *amp, int nx, int ny, double xst, double yst, double xc,
                        double yc, double theta, int sx, int sy);
int mo_defocus_amp_f64(const double *pix, int nx, int ny, float ax, float by, double wavlen,
                       double rprime, float k2maxo, double cs3, double cs5, double *amp);

/* Thermal options of calculate(): lwobble = 1 with nwobble = param[pNWOBBLE] == 1
 * takes the Debye-Waller branch (trlayerDW, autoslic.cpp:766-774, 1039-1160) with
 * temperature = param[pTEMPER]; nwobble > 1 displaces every atom by
 * wobble * gasdev * sqrt(T/300) before the sort (autoslic.cpp:701-713). */
typedef struct {
    const float *wobble;
    int lwobble, nwobble;
    float temperature;
    long *iseed;
} mo_thermal;

double mo_gasdev(long *idum);
int mo_calculate_thermal_f32(float *pix, const float *wave0, const float *param, int natom,
                             const int *Znum, const float *x, const float *y, const float *z,
                             const float *occ, const float *wobble, float ctblength,
                             float ctblengthz, int nmode, int lwobble, long *iseed);
int mo_calculate_thermal_f64(double *pix, const double *wave0, const float *param, int natom,
                             const int *Znum, const float *x, const float *y, const float *z,
                             const float *occ, const float *wobble, float ctblength,
                             float ctblengthz, int nmode, int lwobble, long *iseed);

/* ---- multislice from per-slice potential stacks, and its adjoint (FP64) ----
 * Forward model for one orientation given v[k][ix][iy] (V*Angstrom, the
 * quantity trlayer accumulates, autoslic.cpp:950-984), k = 0..nslices-1:
 *   e_k = exp(i sigma v_k);  t_k = K[M] e_k   (2/3 band limit, autoslic.cpp:999-1009)
 *   u_k = psi_{k-1} t_k;     psi_k = K[p] u_k (propagator, slicelib.cpp:811-849)
 *   phi_d = K[X_d] psi_S;    I_d = |phi_d|^2  (free-space step of mo_defocus_*)
 * with K[m] f = ifft(m fft(f))/(nx ny) in the cfpix convention and psi_0 = 1.
 * Loss L = sum_d sum_px (I_d - T_d)^2.  The adjoint returns dL/dv_k. */
typedef struct {
    int nx, ny;
    float ax, by, v0, deltaz, ctiltx, ctilty;
    int nslices;
    float aobj;          /* objective aperture, rad (0: none) */
    double cs3, cs5;     /* Angstrom */
} mo_stack_params;

int mo_stack_images_f64(const mo_stack_params *p, const double *v, int ndef,
                        const double *rprime, double *images);
double mo_stack_loss_f64(const mo_stack_params *p, const double *v, int ndef,
                         const double *rprime, const float *target);
int mo_stack_adjoint_f64(const mo_stack_params *p, const double *v, int ndef,
                         const double *rprime, const float *target, double *grad, double *loss);
/* Central finite differences of the loss at nvox voxels vox[q] = {k, ix, iy}
 * (k 0-based slice), step h_rel * max(1, |v|), on nthreads threads. */
int mo_stack_fd_f64(const mo_stack_params *p, const double *v, int ndef, const double *rprime,
                    const float *target, int nvox, const int *vox, double h_rel, int nthreads,
                    double *fd);

#ifdef __cplusplus
}
#endif

#endif
