/*
 * msk.h -- C ABI of the GB300 multislice library (libmsk.so).
 *
 * Drop-in for the hot path of timg021/UTR_public's MsctKirkland: Kirkland's
 * autoslic multislice (TemsimLibrary/autoslic.cpp) and the per-orientation
 * loop around it (TemsimLibrary/autosliccmd.cpp), with FFTW replaced by
 * hand-written sm_103a kernels.  Plain pointers and sizes only.
 *
 * Conventions shared by every entry point:
 *   - complex grids are interleaved float pairs (re, im), x-major: element
 *     (ix, iy) at index iy + ix*ny, as the reference's cfpix stores them
 *     (TemsimLibrary/cfpix.hpp:117,133);
 *   - intensity images are float [nx][ny] in the same order;
 *   - the return value is MSK_OK or a negative status; the reference calls
 *     exit(0) in the corresponding cases (autoslic.cpp:258-262, 288-299,
 *     734-739; slicelib.cpp:2847-2851) -- this library returns instead;
 *   - a context owns one CUDA device, one stream and every device buffer;
 *     calls on one context must come from one host thread at a time.
 *   - grid sizes nx, ny: powers of two from 16 to 4096.
 */
#ifndef MSK_H
#define MSK_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct msk_context msk_context;

enum {
    MSK_OK = 0,
    MSK_EBADSIZE = -1,     /* nx, ny < 1 or ax, by < 0                   (autoslic.cpp:258-262) */
    MSK_EBOX = -2,         /* an atom outside [0,ctblength]^2 x [0,ctblengthz] (autoslic.cpp:288-299) */
    MSK_EZSORT = -3,       /* sorted z outside [0, ctblengthz]           (autoslic.cpp:734-739) */
    MSK_EZNUM = -4,        /* atomic number outside 1..103               (slicelib.cpp:2847-2851) */
    MSK_ENOMEM = -5,       /* device or host allocation failed */
    MSK_EUNSUPPORTED = -6, /* grid size or mode this library does not provide */
    MSK_ECUDA = -7,        /* a CUDA call failed; msk_last_error() has the text */
    MSK_EINVAL = -8,       /* bad argument (null pointer, negative count, ...) */
    MSK_ETOOLARGE = -9     /* beyond the fixed scratch of msk_calculate_static */
};

/* param[] offsets read by autoslic::calculate (slicelib.hpp:142-240). */
enum {
    MSK_pXCTILT = 9, MSK_pYCTILT = 10, MSK_pENERGY = 16, MSK_pOAPERT = 17, MSK_pDELTAZ = 30,
    MSK_pAX = 101, MSK_pBY = 102, MSK_pNX = 104, MSK_pNY = 105, MSK_pNWOBBLE = 111,
    MSK_pTEMPER = 120
};

/* Create a context on CUDA device `device`.  Replaces the one-time FFTW plan
 * set-up of cfpix::init (cfpix.cpp:205-264); no FFT plan is shared between
 * contexts or threads. */
int msk_create(int device, msk_context **ctx);
void msk_destroy(msk_context *ctx);
/* Text of the last failure on this context ("" if none). */
const char *msk_last_error(const msk_context *ctx);
const char *msk_status_string(int status);

/* autoslic::calculate, coherent branch (autoslic.hpp:166-169,
 * autoslic.cpp:209-869 with lpartl = lbeams = lcross = 0).
 *   pix     out: complex nx*ny exit wave (resized and overwritten in the reference)
 *   wave0   in:  complex nx*ny incident wave (autoslic.cpp:365)
 *   param   in:  float[>=121]; reads pAX, pBY, pNX, pNY, pENERGY, pDELTAZ,
 *                pXCTILT, pYCTILT (autoslic.cpp:238-252)
 *   Znum, x, y, z, occ, wobble: natom atoms (read only; sorted copies are
 *                made internally, autoslic.cpp:689-724)
 *   ctblength, ctblengthz: the box (autoslic.cpp:288-303)
 *   nmode:  0 multislice; 1, 2 transmission only (autoslic.cpp:783)
 *   lwobble: 1 takes calculate()'s thermal branches (autoslic.cpp:701-713,
 *            766-774) with nwobble = param[pNWOBBLE], T = param[pTEMPER] and
 *            wobble[] = rms displacement at 300 K per atom:
 *              nwobble == 1: Debye-Waller damping exp(-B k^2/4) of every slice's
 *                potential (trlayerDW, autoslic.cpp:1039-1160), B averaged over
 *                wobble[0 .. na-1] of the caller's order as the reference does;
 *              nwobble > 1: every atom displaced by wobble * gasdev(iseed) *
 *                sqrt(T/300) in x, y, z before the sort; *iseed advances.  gasdev
 *                is this library's (the reference's lives in the XArrayLibrary,
 *                which is not part of it): two steps of the 64-bit LCG
 *                (6364136223846793005, 1442695040888963407), Box-Muller from the
 *                top 53 bits.
 *   iseed:   the displacement seed (nwobble > 1 only; may be NULL otherwise)
 * Host pointers.  Blocks until the result is in pix. */
int msk_calculate(msk_context *ctx, float *pix, const float *wave0, const float *param,
                  int natom, const int *Znum, const float *x, const float *y, const float *z,
                  const float *occ, const float *wobble, float ctblength, float ctblengthz,
                  int nmode, int lwobble, long *iseed);

/* One tilt series as MsctKirkland produces it (MultisliceT.cpp:398-448 driving
 * autosliccmd.cpp:711-1224 per orientation): for every orientation, rotate
 * the specimen about z then y' (autosliccmd.cpp:727-748), remove atoms that
 * leave the box (the reference's own rule, autosliccmd.cpp:791-820), for
 * every thermal configuration run calculate() from a plane wave, propagate
 * the exit wave to every detector defocus and record |psi|^2, averaged over
 * configurations in configuration order (autosliccmd.cpp:1205-1224).
 * The free-space step is this library's definition of XArray2DFFT::FresnelA
 * (autosliccmd.cpp:1060,1087), whose source is not part of the reference:
 *   Psi = fft(psi) (cfpix convention), multiply by exp(-i chi) inside the
 *   objective aperture k^2 < (aobj/lambda)^2 (everywhere if aobj == 0), with
 *   chi = pi lambda R k^2 + (pi/2) cs3 lambda^3 k^4 + (pi/3) cs5 lambda^5 k^6
 *       + (pi/2) lambda astig ((kx^2 - ky^2) cos 2a + 2 kx ky sin 2a),
 *   R = defocus - ctblengthz/2 (autosliccmd.cpp:1060), chi in double and
 *   reduced modulo 2 pi, then ifft / (nx*ny) and I = |psi|^2. */
typedef struct {
    int nx, ny;            /* grid */
    float ctblength;       /* field of view = box edge in x and y, Angstrom */
    float ctblengthz;      /* box depth, Angstrom */
    float v0;              /* beam energy, keV */
    float deltaz;          /* slice thickness, Angstrom */
    float aobj;            /* objective aperture semi-angle, rad (0: none) */
    double cs3, cs5;       /* spherical aberrations, Angstrom */
    double astig, astig_angle;  /* two-fold astigmatism, Angstrom and rad */
    double dxc, dyc, dzc;  /* rotation centre shift from the box centre, Angstrom */
    int nmode;             /* as in msk_calculate */
    int max_batch;         /* waves in flight at once (0: as many as memory allows) */
    /* thermal branches, as msk_calculate with nconfig in the role of nwobble:
     * lwobble = 1 and nconfig == 1 damps every slice's potential by the
     * Debye-Waller factor; lwobble = 1 and nconfig > 1 without displacements
     * draws them in the engine, orientation i from the seed `seed - i`, its
     * configurations in order from that sequence */
    int lwobble;
    float temperature;     /* K */
    const float *wobble;   /* rms displacement at 300 K per atom (host; lwobble = 1) */
    long seed;
    /* incident wave: 0 a plane wave; else a spherical wave from a point source
     * R1 Angstrom before the box centre (autosliccmd.cpp:650-689) */
    double R1;
    /* image plane (autosliccmd.cpp:1119-1143): rotation[d] (radians; NULL: none)
     * about the optic axis through the box centre + (dxc, dyc), then a shift by
     * (xshift, yshift) Angstrom rounded to whole pixels, both applied to the
     * propagated amplitude of detector plane d before |psi|^2.  The reference
     * calls the missing XArrayLibrary for them; this library's definitions:
     * Catmull-Rom bicubic interpolation, out(p) = in(c + R(-theta)(p - c)) with
     * the atom rotation's R, and values outside the image taken as the mean of
     * the 5-pixel border (per real and imaginary part). */
    const double *rotation;
    double xshift, yshift;
} msk_series;

/*   natom atoms: Znum, x, y, z, occ (host)
 *   nangles orientations: angleZ[i], angleY[i] in radians (host)
 *   ndefocus defoci in Angstrom from the box centre (host)
 *   nconfig >= 1 thermal configurations; displacements (host, may be NULL
 *     when nconfig == 1): float[nconfig][3][natom] added to x, y, z after the
 *     rotation (the reference's calculate() adds its random displacement to
 *     the rotated coordinates, autoslic.cpp:701-713)
 *   images   out: float[nangles][ndefocus][nx][ny]; host or device pointer
 *            (page-locked host memory the GPU can address receives each
 *            batch's images while the next batch runs, written by the GPU
 *            through the mapped address; other host memory gets one copy
 *            at the end)
 *   exitwaves out (may be NULL): complex [nangles][nconfig][nx][ny]; host or
 *     device pointer
 *   kept     out (may be NULL): int[nangles*nconfig], atoms inside the box */
int msk_tilt_series(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                    const float *x, const float *y, const float *z, const float *occ,
                    int nangles, const double *angleZ, const double *angleY, int ndefocus,
                    const double *defocus, int nconfig, const float *displacements,
                    float *images, float *exitwaves, int *kept);

/* One detector plane of one orientation (msk_tilt_series_planes,
 * msk_tilt_series_batch). */
typedef struct {
    double defocus;       /* Angstrom from the box centre */
    double rotation;      /* about the optic axis, radians (the image-plane rotation) */
    double astig;         /* two-fold astigmatism, Angstrom */
    double astig_angle;   /* radians */
} msk_plane;

/* Many specimens in one call: MultisliceT.cpp:398-448 run for each specimen,
 * with its own atoms, box, grid and orientations; the common beam, slicing,
 * lens, incident wave (R1), image plane (rotation, xshift, yshift), thermal
 * and defocus settings come from `s` (its nx, ny, ctblength, ctblengthz,
 * max_batch and wobble are not read).  With lwobble = 1 and one configuration
 * per orientation the Debye-Waller branch, with several (nconfig) random
 * displacements, each with the specimen's wobble: msk_tilt_series with that
 * nconfig and no displacements.  All specimens' tables, atoms,
 * waves and images live in one device arena (in waves of specimens when they
 * do not fit); specimens run on concurrent streams, longest first.  With
 * flags & MSK_BATCH_GRAPH the launches are captured into one CUDA graph and
 * launched once.  Results equal msk_tilt_series (msk_tilt_series_planes for
 * a specimen with its own plane lists) per specimen. */
typedef struct {
    int natom;
    const int *Znum;
    const float *x, *y, *z, *occ;
    int nx, ny;                       /* this specimen's grid */
    float ctblength, ctblengthz;      /* this specimen's box, Angstrom */
    int nangles;
    const double *angleZ, *angleY;    /* radians */
    float *images;   /* out: float[nangles][ndefocus][nx][ny], host or device */
    int *kept;       /* out (may be NULL): int[nangles] (see nconfig) */
    const float *wobble;  /* rms displacement at 300 K per atom (host; s->lwobble = 1) */
    int nconfig;          /* thermal configurations per orientation (0, 1: one), images
                           * averaged; kept then holds int[nangles * nconfig] */
    const float *displacements;  /* float[nconfig][3][natom] added to x, y, z after the
                                  * rotation (host, may be NULL), as msk_tilt_series; NULL
                                  * with nconfig > 1 needs s->lwobble = 1 (drawn in the
                                  * engine) */
    float *exitwaves;  /* out (may be NULL): complex [nangles][nconfig][nx][ny], host or
                        * device, as msk_tilt_series */
    const int *plane_off;     /* (may be NULL) this specimen's own detector planes per
                               * orientation, as msk_tilt_series_planes takes them:
                               * orientation a images planes [plane_off[a], plane_off[a+1])
                               * of `planes`, shifted by shifts[2a], shifts[2a+1] Angstrom
                               * (NULL: none); images then float[plane_off[nangles]][nx][ny].
                               * The call's ndefocus, defocus and s's rotation, astig,
                               * astig_angle, xshift and yshift are not read for it. */
    const msk_plane *planes;
    const double *shifts;
} msk_specimen;

enum { MSK_BATCH_GRAPH = 1 };

int msk_tilt_series_batch(msk_context *ctx, const msk_series *s, int nspec,
                          const msk_specimen *spec, int ndefocus, const double *defocus,
                          int flags);

/* The tilt series with its own detector planes per orientation, as
 * MsctKirkland's orientation files give them (MultisliceT.cpp:264-285; see
 * msk_read_orientations): orientation i images planes [plane_off[i],
 * plane_off[i+1]) of `planes`, its images shifted by shifts[2i], shifts[2i+1]
 * Angstrom (NULL: none); images[k] (float[plane_off[nangles]][nx][ny], host or
 * device) is the image of plane k.  The lens settings other than astigmatism
 * (aobj, cs3, cs5) and everything else come from `s`; its astig, astig_angle,
 * rotation, xshift and yshift are not read.  Planes with equal parameters in
 * different orientations share one free-space table and pass. */
int msk_tilt_series_planes(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                           const float *x, const float *y, const float *z, const float *occ,
                           int nangles, const double *angleZ, const double *angleY,
                           const int *plane_off, const msk_plane *planes, const double *shifts,
                           int nconfig, const float *displacements, float *images,
                           float *exitwaves, int *kept);

/* calculate() without any allocation -- no counterpart in the reference.
 * For callers that cannot allocate device memory (a plug-in inside a host
 * framework that owns all device memory through its own pool, or a loop that
 * cannot take cudaMalloc's latency and implicit synchronisation).  The
 * arguments and result of msk_calculate's coherent branch: no context, and no
 * thermal branch (msk_calculate's wobble, lwobble and iseed are not taken);
 * plus the CUDA stream to run on (NULL: the legacy default stream); host
 * pointers; blocks until pix is written.  Its device scratch is a fixed
 * 8.07 MiB array in this library, held by every GPU that loads it until the
 * process exits; no call allocates device memory (a buffer that would have to
 * grow fails the call with MSK_ENOMEM instead; msk_device_allocations counts).
 * Limits: nx*ny <= 512*512, natom <= 65536, <= 4096 slices; beyond them it
 * returns MSK_ETOOLARGE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  Every call reuses the same array and
 * leaves its contents behind (each call initialises what it reads), so calls
 * that overlap on the GPU -- from two host threads or on two streams -- race
 * and corrupt each other's results: serialise them. */
int msk_calculate_static(void *stream, float *pix, const float *wave0, const float *param,
                         int natom, const int *Znum, const float *x, const float *y,
                         const float *z, const float *occ, float ctblength, float ctblengthz,
                         int nmode);

/* The schedule the column-pass tuner chose for a grid on a device -- no
 * counterpart in the reference (whose FFTW planning, cfpix.cpp:225-228, is
 * internal to FFTW).  pass: 0 band limit, 1 propagator, 2 free-space step,
 * 3 Debye-Waller damping.  info[0] = variant (MSK_COL_TILE's numbering),
 * info[1] = points a thread holds in the FFT's first stage (32 or 16),
 * info[2] = columns per CTA.  MSK_EINVAL until that pass has run on that grid. */
int msk_column_plan(int device, int nx, int ny, int pass, int *info);

/* The schedule the row tuner chose for a grid on a device -- no counterpart in
 * the reference (FFTW planning, as above).  pass: 0 the transmit (the wave's
 * and the transmission's row transforms and their product; both the wave and
 * the scattered form).  info[0] = variant (MSK_ROW_PLAN's numbering: 0 = 32
 * points a thread in 64-thread CTAs, 1 = 32 points in 128-thread CTAs, 2 = 16
 * points in 128-thread CTAs), info[1] = points a thread, info[2] = rows per CTA.
 * MSK_EINVAL until the transmit has run on that grid. */
int msk_row_plan(int device, int nx, int ny, int pass, int *info);

/* Device allocations (cudaMalloc) this library has made in this process so far,
 * over every context -- no counterpart in the reference; lets a caller check
 * that a run of msk_calculate_static calls allocated nothing. */
long long msk_device_allocations(void);

/* Use the caller's CUDA stream (a cudaStream_t) for this context's work
 * instead of the context's own; NULL restores the context's stream. */
int msk_set_stream(msk_context *ctx, void *stream);

/* Per-kernel accounting: with profiling on, every launch is bracketed by CUDA
 * events on the context's stream and its algorithmic HBM bytes are counted
 * (the bytes a launch must move at minimum: a complex64 grid read or written
 * is 8 bytes per pixel).  msk_profile(ctx, 1) clears the counters and starts;
 * msk_profile(ctx, 0) stops.  msk_profile_read fills up to max entries and
 * returns how many kinds have counts; host<->device copies made by the
 * library appear as "copy_h2d" / "copy_d2h" (launches = copies, ms = 0). */
typedef struct {
    char name[32];
    long long launches;
    double ms;      /* summed event time */
    double bytes;   /* summed algorithmic bytes */
} msk_kernel_stat;
int msk_profile(msk_context *ctx, int enable);
int msk_profile_read(msk_context *ctx, msk_kernel_stat *out, int max);

/* The same tilt series (same arguments except exit waves, same results within
 * rounding) computed as a direct GPU port of the reference's loop would:
 * orientation by orientation (MultisliceT.cpp:403-448 runs one host thread
 * per orientation), per slice an atomic scatter of the potential
 * (autoslic.cpp:950-984), unfused element-wise kernels and library 2D FFTs
 * (cuFFT, loaded at run time: MSK_EUNSUPPORTED if it cannot be), a
 * synchronisation after every orientation.  The comparison form for the
 * batched msk_tilt_series. */
int msk_tilt_series_per_angle(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                              const float *x, const float *y, const float *z, const float *occ,
                              int nangles, const double *angleZ, const double *angleY,
                              int ndefocus, const double *defocus, int nconfig,
                              const float *displacements, float *images, int *kept);

/* Multislice from given per-slice projected potentials, and its adjoint.
 * The slice loop of calculate() (autoslic.cpp:838-861: transmission
 * exp(i sigma v_k) band-limited to 2/3 kmax, wave *= trans, Fresnel
 * propagator) with v_k supplied instead of splatted from atoms, from a plane
 * wave psi_0 = 1, then the free-space step of msk_tilt_series to each
 * detector plane and I = |psi|^2.  The adjoint returns dL/dv for the image
 * misfit L = sum over units, planes, pixels of (I - target)^2.  With
 * checkpoint 0 the forward pass keeps every wave and transmission (2S + 4
 * grids per unit) when at least min(nunits, 32) units fit in memory at once,
 * and the backward pass recomputes nothing; otherwise (and with checkpoint
 * K > 0) it keeps the wave every K slices (8 for checkpoint 0) and recomputes
 * the waves inside a block from its checkpoint.  The reference has no
 * adjoint. */
typedef struct {
    int nx, ny;            /* grid */
    float ax, by;          /* cell size, Angstrom (param[pAX], param[pBY]) */
    float v0;              /* beam energy, keV */
    float deltaz;          /* slice thickness, Angstrom */
    float ctiltx, ctilty;  /* crystal tilt, rad (param[pXCTILT], param[pYCTILT]) */
    float aobj;            /* objective aperture semi-angle, rad (0: none) */
    double cs3, cs5;       /* spherical aberrations, Angstrom */
    int nslices;           /* slices per stack (>= 1) */
    int checkpoint;        /* slices per checkpoint block of the adjoint (0: keep all) */
    int max_batch;         /* units in flight at once (0: as many as memory allows) */
} msk_stack;

/*   nunits independent stacks (orientations): v float[nunits][nslices][nx][ny]
 *     in the potential units of the atom path (phase = sigma * v), host or device
 *   ndefocus detector planes at distance defocus[d] (Angstrom) past the exit face
 *   images out: float[nunits][ndefocus][nx][ny], host or device */
int msk_stack_images(msk_context *ctx, const msk_stack *s, int nunits, const float *v,
                     int ndefocus, const double *defocus, float *images);

/*   target: float[nunits][ndefocus][nx][ny], host or device (ndefocus >= 1)
 *   grad out: float[nunits][nslices][nx][ny] = dL/dv, host or device
 *   loss out (may be NULL): L, summed in double in a fixed order */
int msk_adjoint(msk_context *ctx, const msk_stack *s, int nunits, const float *v,
                      int ndefocus, const double *defocus, const float *target, float *grad,
                      double *loss);

/* The projected potential of every slice of every orientation of a tilt
 * series, as the atom path splats it before the transmission exp(i sigma v)
 * (trlayer, autoslic.cpp:917-984): orientations, box and slicing as in
 * msk_tilt_series (s->nx, ny, ctblength, ctblengthz, deltaz, v0, dxc..dzc,
 * max_batch are read).  Feeding v to msk_stack_images with defocus
 * d - ctblengthz/2 gives msk_tilt_series's images.
 *   v out: float[nangles][msk_slice_count(deltaz, ctblengthz)][nx][ny],
 *          host or device
 *   kept out (may be NULL): int[nangles], atoms inside the box */
int msk_potential_stack(msk_context *ctx, const msk_series *s, int natom, const int *Znum,
                        const float *x, const float *y, const float *z, const float *occ,
                        int nangles, const double *angleZ, const double *angleY, float *v,
                        int *kept);

/* MsctKirkland's files (the reference reads and writes them through its
 * XArrayLibrary, which is not part of it).  Images are [nx][ny] (iy fastest)
 * and are written with rows along y, x fastest, as the reference transposes
 * its cfpix data before writing (autosliccmd.cpp:1053-1055); little-endian.
 *   GRD (ReadmeMsctKirkland.txt): "DSBB", nx ny (short), xlo xhi ylo yhi zlo zhi
 *        (double; z = the value range), the values (float)
 *   GRC: -5 (short), wavelength (double), nx ny (short), xlo xhi ylo yhi
 *        (double), re im pairs (float)
 *   TIFF32: baseline TIFF, one strip of 32-bit IEEE floats
 * MSK_EINVAL when the file cannot be written. */
int msk_write_grd(const char *path, const float *img, int nx, int ny, double xlo, double xhi,
                  double ylo, double yhi);
int msk_write_grc(const char *path, const float *amp, int nx, int ny, double wavelength,
                  double xlo, double xhi, double ylo, double yhi);
int msk_write_tiff32(const char *path, const float *img, int nx, int ny);

/* MsctKirkland's orientation file (its parameter 17, ".txt" or ".relionnew"):
 * angles[2i], angles[2i+1] = rotations about Z and Y' (degrees) of orientation
 * i; its detector planes [plane_off[i], plane_off[i+1]) with planes[5k..5k+4] =
 * {Z'' rotation (degrees), defocus from the object centre, astigmatism,
 * astigmatism angle (degrees), 0}; shifts[2i], shifts[2i+1] = image shift along
 * x and y.  Call first with null arrays: *nangles and *nplanes receive the
 * counts; then with arrays of those sizes (plane_off: nangles + 1) and the
 * counts as capacities.  ".txt": "//" comment lines, then per line the Z and
 * Y' angles and (Z'' angle, defocus) pairs.  ".relionnew": index, name, x
 * shift, y shift, defocus U, defocus V, astigmatism angle, rot, tilt, psi per
 * line; every number but the astigmatism angle changes sign (the readme's
 * rule); defocus = (U + V)/2, astigmatism = (U - V)/2 (this library's reading;
 * the reference's reader is in the missing XArrayLibrary).  MSK_EINVAL on a
 * malformed file or an unknown extension. */
int msk_read_orientations(const char *path, int *nangles, int *nplanes, double *angles,
                          int *plane_off, double *planes, double *shifts);

/* Number of slice-steps calculate() runs for a box of depth ctblengthz
 * (autoslic.cpp:747-830: zslice = dz, dz + dz, ... while < ctblengthz + dz). */
int msk_slice_count(float deltaz, float ctblengthz);

/* Slice index (0-based) of every atom of a z-sorted list, with the
 * reference's double-precision slice boundaries (autoslic.cpp:756-762). */
int msk_slice_assign(float deltaz, float ctblengthz, int natom, const float *zsorted,
                     int *slice_of_atom);

/* The reference's Shell sort by z (slicelib.cpp:2467-2504), in place: the
 * same permutation as the reference for the same input. */
void msk_sort_by_z(float *x, float *y, float *z, float *occ, int *Znum, int natom);

/* Rotation about z then y' in float (autosliccmd.cpp:727-748), in place. */
void msk_rotate(float ctblength, double dxc, double dyc, double dzc, double angleZ,
                double angleY, int natom, float *x, float *y, float *z);

/* The projected-potential spline table of atomic number Z as the kernels use
 * it (slicelib.cpp:2812-2875): knots[100] (r^2) and coef[100][4] = {y,b,c,d}
 * computed in double.  Returns MSK_EZNUM for Z outside 1..103. */
int msk_potential_table(int Z, double *knots, double *coef);

#ifdef __cplusplus
}
#endif

#endif /* MSK_H */
