/*
 * zorro_gb300 -- C ABI of the GB300 (sm_103a) movie-registration hot path.
 *
 * The entry points below replace, step by step, the body of
 * ``ImageRegistrator.alignImageStack`` in LBEM-CH/zorro (zorro/zorro.py:1569)
 * and the steps it drives.  Each declaration names the reference code it
 * stands for.  All pointers are DEVICE pointers unless stated otherwise,
 * all work is enqueued on ``stream`` (a cudaStream_t passed as void*), and no
 * entry point allocates device memory: scratch space is passed in as
 * ``work``/``work_bytes`` (query the size with the matching *_work_bytes
 * function).  Return value: ZR_OK (0) or a negative ZR_E* code; the message
 * of the last failure on the calling thread is available from
 * zr_last_error().
 *
 * Layouts (row-major, C order):
 *   frames      [N][H][W] raw counts (see zr_frames_t)
 *   spectrum    [K4][C0+4] complex float, column-major: K4 = zr_spectrum_pitch(C1)
 *               columns, column k holding kx = k for 0 <= k <= C1/2 (the half-plane
 *               of a real image); in each column, elements 0..C0-1 are the
 *               Fourier-cropped frequencies ky in FFT order (element C0/2 holds
 *               ky = -C0/2), element C0 holds ky = +C0/2, the rest is padding.
 *   window      [w][w] float, w = 2*max_shift; element (a, b) is the correlation
 *               at shift (y, x) = (a - max_shift, b - max_shift).
 */
#ifndef ZORRO_GB300_H
#define ZORRO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZR_OK 0
#define ZR_EINVAL (-1)   /* invalid argument (ValueError in the reference) */
#define ZR_ECUDA (-2)    /* CUDA runtime error */
#define ZR_ESIZE (-3)    /* size outside what the kernels support */
#define ZR_EWORK (-4)    /* scratch buffer too small */

/* raw pixel types */
#define ZR_F32 0
#define ZR_U8 1
#define ZR_U16 2
#define ZR_F16 3

/* One movie's frames and the per-pixel corrections applied when they are
 * read: v = float32(gain*raw) (zorro.py:3466), v /= gain_divisor when nonzero
 * (zorro.py:3477), v = hot_a*v + hot_b (hotpixFilter, zorro.py:2649). */
typedef struct zr_frames {
  const void* raw;
  int raw_type;
  const float* gain;   /* [H][W] or NULL */
  const float* hot_a;  /* [H][W] or NULL (then hot_b is ignored) */
  const float* hot_b;  /* [H][W] */
  float gain_divisor;  /* 0: none */
  int n_frames, height, width;
  long long frame_stride; /* elements between frames, 0 = height*width */
  /* Frames of several movies in one call (the batched path): frame n reads
   * the maps of movie frame_movie[n] (device array of n_frames ints), which
   * start map_stride elements apart in gain, hot_a and hot_b.  NULL: every
   * frame reads the one [H][W] map set.  zr_gain_sum and zr_shift_sum work on
   * one movie at a time and refuse it. */
  const int* frame_movie;
  long long map_stride;
} zr_frames_t;

/* Hot-pixel filter constants (zorro.py:2595-2649). */
typedef struct zr_hotpix_params {
  double mu, sigma;          /* fitted normal CDF of the unaligned sum */
  float cutoff_lower, cutoff_upper;
  float logistic_k, relax;
  float psf[9];              /* normalised 3x3 detector PSF */
  float neighbour_thres;     /* 0.01 */
  double best_mean;          /* mu / n_frames */
} zr_hotpix_params_t;

/* Peak search constants (locatePeak, zorro.py:1099-1231). */
typedef struct zr_peak_params {
  int sub_pix_reg;           /* subPixReg */
  int bmode;                 /* 0 none, 1 'opti', 2 'conv' */
  int suppress_origin;       /* suppressOrigin */
  int use_mask;              /* maxShift circular mask */
  double conv_sigma_y, conv_sigma_x; /* bmode 2 */
  double opti_lo, opti_hi, opti_xatol; /* 0, 7, 0.01 */
  int opti_maxiter;          /* 15 */
} zr_peak_params_t;

typedef struct zr_peak_result {
  double shift_y, shift_x;   /* in cropped pixels (before the P/C scale) */
  double sigma;              /* 'opti' Gaussian sigma */
  float corr, peaksig, origin;
  int cy, cx;                /* integer peak position in the window */
  int flags;                 /* bit0: sub-pixel patch hit the window edge */
  int nfev;
} zr_peak_result_t;

/* Per-frame shift applied by applyShifts (zorro.py:1774 ->
 * zorro_util.py:341-379): np.roll by (roll_y, roll_x), given reduced modulo
 * the frame height and width (0 <= roll_y < H, 0 <= roll_x < W), then the
 * separable 3x3 Lanczos kernel ky (x) kx with reflect boundaries (identity
 * when apply == 0). */
typedef struct zr_shift {
  int roll_y, roll_x;
  int apply;
  float ky[3], kx[3];
} zr_shift_t;

/* Dose-filter constants (doseFilter, zorro.py:2375-2452). */
typedef struct zr_dose_params {
  float crit_a, crit_b, crit_c;  /* critical-dose curve */
  float cutoff_order;            /* 32 */
  float voltage_scaling;         /* sqrt(kV/300) */
  float inv_ps_x, inv_ps_y;      /* 1/(P*pixelsize_A) */
  int normalize;                 /* 'dosenorm' */
} zr_dose_params_t;

int zr_version(void);
int zr_last_error(char* buf, size_t len);

/* Number of kernels this library has launched in the process (instrumentation;
 * no counterpart in the reference). */
unsigned long long zr_launch_count(void);

/* One-time per-device setup (twiddle table).  Replaces the FFTW planning in
 * zorro_util.py:966-1066 (pyFFTWPlanner). */
int zr_init(int device);

/* ---- gain and hot pixels: hotpixFilter, zorro.py:2497-2672 ---- */

/* unaligned_sum[y][x] = sum over n (in frame order, float32) of the gain-
 * corrected frames (zorro.py:2529); *total (double, accumulated) += sum of
 * all pixels of unaligned_sum.  Hot-pixel maps in ``frames`` are ignored. */
int zr_gain_sum(const zr_frames_t* frames, float* unaligned_sum, double* total, void* stream);

/* np.histogram(values, edges) for unit-width bins first_edge + i
 * (zorro.py:2533-2534).  counts[nbins] is accumulated, not cleared. */
int zr_histogram(const float* values, long long n, double first_edge, int nbins,
                 unsigned int* counts, void* stream);

/* The float32 thresholds of the dead/hot counts (zorro.py:2595-2601): a
 * float32 value s is counted dead when s < *s_dead and hot when s >= *s_hot,
 * exactly when the float64 quotient (s - mu) / sigma lies below cutoff_lower
 * or above cutoff_upper (*s_hot is NaN when no value is above).  sigma >= 0.
 * Host code (bisection over the ordered float32 values). */
int zr_hotpix_thresholds(double mu, double sigma, float cutoff_lower, float cutoff_upper, float* s_dead,
                         float* s_hot);

/* The logistic masks, PSF fill and neighbour fill of zorro.py:2595-2649,
 * folded into per-pixel affine maps hot_a (logisticMask) and hot_b
 * (singletonOutlierMask*psfFiltMean + neighbourFilt).  counts3 (accumulated)
 * receives guessDeadpix, guessHotpix and neighborPix.  ``work`` holds
 * zr_hotpix_work_bytes() bytes. */
size_t zr_hotpix_work_bytes(int height, int width);
int zr_hotpix_maps(const float* unaligned_sum, int height, int width, int n_frames,
                   const zr_hotpix_params_t* params, float* hot_a, float* hot_b,
                   unsigned int* counts3, void* work, size_t work_bytes, void* stream);

/* ---- movie input: MRC mode 101 (zorro.loadData, zorro.py:3414-3425, read
 * through mrcz) ----
 * frames[n][y][x] (uint8) = 4-bit pixel x of row y of frame n in ``packed``
 * ([n_frames][height][(width+1)/2] bytes, the first pixel of each byte in its
 * low 4 bits, rows padded to whole bytes). */
int zr_unpack_u4(const void* packed, int n_frames, int height, int width, void* frames, void* stream);

/* ---- Fourier binning: binStack(binKernel='fourier'), zorro.py:1826-1904 ----
 * out[n] (float, [Hb][Wb]) = real(IFFT_unscaled(crop(FFT(frame n))) / (Hb Wb)),
 * the crop keeping rows [0, Hb/2) and [H - Hb/2, H) and columns likewise; the
 * frames are read with their gain (hot-pixel maps are not applied: the
 * reference bins before its hot-pixel filter).  Hb and Wb even; every side
 * in 513..8192 (Bluestein transforms of 2048..16384 points).  work:
 * zr_bin_work_bytes(H, W, Hb, Wb) bytes. */
size_t zr_bin_work_bytes(int H, int W, int Hb, int Wb);
int zr_bin_fourier(const zr_frames_t* frames, int Hb, int Wb, float* out, void* work, size_t work_bytes,
                   void* stream);

/* ---- forward spectra: xcorrnm2_tri, zorro.py:814-925 ---- */

/* sums[n] (double, accumulated) += sum of the corrected frame n over
 * [0,H)x[0,W).  Used to subtract each frame's mean before the transform
 * (the masked normalised correlation with a binary mask does not change when
 * a constant is subtracted inside the mask). */
int zr_frame_sums(const zr_frames_t* frames, double* sums, void* stream);

int zr_spectrum_pitch(int C1);
long long zr_spectrum_elems(int C0, int C1);
size_t zr_spectra_work_bytes(int height, int n_frames, int C1);

/* Fourier-cropped spectra of frames [frame0, frame0+n_frames): G = FFT(m*I),
 * S = FFT((m*I)^2) at P0 x P1, cropped to C0 x C1 (zorro.py:875-914).  I is
 * the corrected frame minus mean_sub[n] (NULL: 0), zero-padded to P0 x P1;
 * m is ``mask`` ([P0][P1], NULL: ones on [0,H)x[0,W), the padStack mask,
 * zorro.py:1943-1949).  mode 1 transforms the mask itself into G (S unused),
 * zorro.py:814-825.  G and S point at the spectrum of frame ``frame0``. */
int zr_spectra(const zr_frames_t* frames, const float* mask, const double* mean_sub, int frame0,
               int n_frames, int mode, int P0, int P1, int C0, int C1, void* G, void* S,
               void* work, size_t work_bytes, void* stream);

/* ---- masked normalised cross-correlation: mnxc2, zorro.py:1014-1097 ---- */

/* Scratch of the correlation passes: (2*max_shift + 1) rows of
 * zr_spectrum_pitch(C1) complex values per job of a wave; any size from one
 * job up works (larger means fewer, bigger waves). */
size_t zr_xcorr_work_bytes(int n_jobs, int C1, int max_shift);

/* The frame-only terms of mnxc2, windowed: for every frame n the windows of
 * CorrTM (template mask), CorrBM (base mask), the two Denominator IFFTs, and
 * the maskProduct; terms is [4N+1][w][w] (order CTM[0..N), CBM, DT, DB, MP).
 * zorro.py:1034-1057 and 826-835.  G, S: N spectra each; GM: mask spectrum. */
int zr_xcorr_terms(const void* G, const void* S, const void* GM, int N, int C0, int C1,
                   int max_shift, float* terms, void* work, size_t work_bytes, void* stream);

/* The correlation windows C of pairs (I, J) (template I, base J):
 * numerator IFFT of G_J conj(G_I), combined with the terms as in
 * zorro.py:1061-1092 (Denom clipped to >= 1), ifftshift-cropped to the
 * +/-max_shift window.  pairs is [M][2] int (I, J). */
int zr_xcorr_pairs(const void* G, const float* terms, const int* pairs, int M, int N, int C0, int C1,
                   int max_shift, float* cwin, void* work, size_t work_bytes, void* stream);

/* zr_xcorr_pairs without a work buffer.  This entry point has no counterpart
 * in the reference.  It is for callers that may not allocate device memory
 * when they call in: a host process that owns the whole device-memory budget
 * and forbids allocation inside its callbacks, or a caller that keeps every
 * allocation out of its per-request loop.  The scratch is a device array of
 * ZR_XCORR_STATIC_SCRATCH bytes compiled into the library; the pairs run in
 * waves of floor(ZR_XCORR_STATIC_SCRATCH / (2*max_shift * K4 * 8)) pairs
 * (K4 = zr_spectrum_pitch(C1)), and a size whose single pair does not fit
 * returns ZR_ESIZE.  Nothing in the scratch has to start at zero.
 * - The first call on each device looks the array's address up
 *   (cudaGetSymbolAddress, with that device current); make that first call
 *   before any stream capture on the device.
 * - Every call on a device shares the one array: calls that overlap in time
 *   (different streams or threads with no ordering between them) race on it
 *   and give wrong results.  Order them on one stream.
 * Results are those of zr_xcorr_pairs. */
#define ZR_XCORR_STATIC_SCRATCH (16u << 20)
int zr_xcorr_pairs_noalloc(const void* G, const float* terms, const int* pairs, int M, int N, int C0, int C1,
                           int max_shift, float* cwin, void* stream);

/* Half-precision spectra (the mixed-precision form of the path; the
 * reference stores complex64): spectrum n of ``spectra`` ([n_spectra][se]
 * complex float) is written to ``out`` as __half2 times scales[n], a power
 * of two with max(|re|, |im|) * scales[n] < 2^15.  work: n_spectra * 4
 * bytes.  The _half correlation passes read such spectra (G, S and GM with
 * scales [N] G, [N] S, [1] GM; the pair pass uses the G scales), undo the
 * scales exactly, and otherwise compute what zr_xcorr_terms / zr_xcorr_pairs
 * compute, in float. */
int zr_pack_half(const void* spectra, int n_spectra, long long se, void* out, float* scales, void* work,
                 size_t work_bytes, void* stream);
int zr_xcorr_terms_half(const void* G, const void* S, const void* GM, const float* scales, int N, int C0, int C1,
                        int max_shift, float* terms, void* work, size_t work_bytes, void* stream);
int zr_xcorr_pairs_half(const void* G, const float* scales, const float* terms, const int* pairs, int M, int N,
                        int C0, int C1, int max_shift, float* cwin, void* work, size_t work_bytes, void* stream);

/* triMode 'refine' (xcorrnm2_tri, zorro.py:934-954): frame I (I < N-1) is
 * correlated with the template of all frames but I.
 * zr_refine_spectra: templates[n] = (sum_m G[m] - G[n]) / N for every n (the
 * reference's conj(sumFFT - baseImageFFT[I]) / N enters as A conj(B)).
 * zr_refine_terms: the frame terms with CorrTM and DenomT of every slot n
 * replaced by the template's, (sum_m term_m - term_n) / N (they are linear in
 * the template spectra); out is [4N+1][w][w] like terms.
 * zr_xcorr_refine: the N-1 windows of frame I against template I, combined
 * with refine_terms as mnxc2 combines any pair; cwin is [N-1][w][w]. */
int zr_refine_spectra(const void* G, int N, int C0, int C1, void* templates, void* stream);
int zr_refine_terms(const float* terms, int N, int max_shift, float* out, void* stream);
int zr_xcorr_refine(const void* G, const void* templates, const float* refine_terms, int N, int C0, int C1,
                    int max_shift, float* cwin, void* work, size_t work_bytes, void* stream);

/* ---- peak search: locatePeak, zorro.py:1099-1231 ---- */
int zr_locate_peaks(const float* cwin, int M, int max_shift, const zr_peak_params_t* params,
                    zr_peak_result_t* results, void* stream);

/* ---- preShift peak search on uncropped planes: locatePeak with preShift,
 * zorro.py:1089-1092 (no crop), 1148-1168 (rolled mask) ----
 * ``planes`` are n whole C x C correlation planes, ifftshifted (the output of
 * zr_xcorr_pairs with max_shift = C/2).  The host runs the bounded Brent
 * search over sigma for every plane of a batch in lock step.
 *
 * zr_full_prepare: origin[p] = the plane's value at (C/2, C/2); with
 * suppress_origin the stencil of zorro.py:1082-1083 replaces it (in place);
 * mean[p] = the plane's mean afterwards.
 *
 * zr_full_filter: for the planes listed in sel[0..n_sel), the separable
 * Gaussian filter (axis 0, then axis 1, 'reflect' borders) with the taps
 * weights[p][a][0 .. 2*radius[p][a]] of axis a (radius <= 64; 2 x 129 floats
 * a plane), kept in filtered[p] when ``filtered`` is not NULL; stats[p] =
 * (sum (F - mean[p]), sum (F - mean[p])^2, max F), summed in a fixed order.
 *
 * zr_full_peaks: for the listed planes, the maxShift disc about (C/2, C/2)
 * np.roll-ed by rolls[p] = (ry, rx): argmax of filtered * disc (first index
 * on ties), the peak significance over the disc, and the sub-pixel step of
 * zr_locate_peaks on the filtered plane (unfiltered value at the integer
 * fallback); results[p] gets sigma[p] and nfev[p] as given.
 * work: zr_full_work_bytes(n_planes, C) bytes. */
int zr_full_prepare(float* planes, int n, int C, int suppress_origin, float* origin, float* mean, void* stream);
size_t zr_full_work_bytes(int n_planes, int C);
int zr_full_filter(const float* planes, int n_planes, int C, const int* sel, int n_sel, const float* weights,
                   const int* radius, const float* mean, float* filtered, double* stats, void* work,
                   size_t work_bytes, void* stream);
int zr_full_peaks(const float* planes, const float* filtered, int n_planes, int C, const int* sel, int n_sel,
                  int max_shift, const int* rolls, const float* mean, const float* origin, const double* sigma,
                  const int* nfev, int sub_pix_reg, zr_peak_result_t* results, void* work, size_t work_bytes,
                  void* stream);

/* ---- shift and sum: applyShifts + lazyFouRingCorr sums, zorro.py:1734-1808, 2237-2238 ---- */
/* image_sum = sum_n shifted frame n (float32, frame order); even_sum/odd_sum
 * likewise over even/odd n (either may be NULL); ``aligned`` [N][H][W]
 * receives the shifted frames when not NULL.  shifts: device array [N]. */
int zr_shift_sum(const zr_frames_t* frames, const zr_shift_t* shifts, float* image_sum,
                 float* even_sum, float* odd_sum, float* aligned, void* stream);

/* ---- tiled FRC: tiledFRC, zorro.py:2246-2310 + rotmean, zorro_util.py:147-224 ---- */

size_t zr_frc_work_bytes(int n_tiles, int box);
/* offsets: device int array [n_tiles][2] (y, x) of the box x box tiles.  frc2d
 * [box][box] receives the fftshifted, DC-normalised 2-D FRC; frc [nrings]
 * (double) its rotational mean. */
int zr_tiled_frc(const float* even, const float* odd, int height, int width, int box,
                 const int* offsets, int n_tiles, float* frc2d, double* frc, int nrings,
                 void* work, size_t work_bytes, void* stream);

/* ---- drift solve: shiftsSolver, zorro.py:1260-1567 (host only) ---- */

/* Exact weighted L1 regression on the host: x = argmin sum_i w_i |(A x)_i - b_i|,
 * the objective of shiftsSolver (zorro_util.py:849-851), which the reference
 * minimises with scipy.optimize.basinhopping (zorro.py:1415,1422).  A, b, w, x
 * are HOST arrays (A row-major [m][n]).  *status: 0 optimum found inside
 * [lo, hi]; 4 optimum found but outside the box (the caller solves the bounded
 * problem instead). */
int zr_l1_solve(const double* A, const double* b, const double* w, int m, int n, double lo, double hi,
                double* x, int* status);

/* Logistic fit of the peak-significance CDF: the minimisation in
 * cdfLogisticCurve (zorro.py:1981-2022) of the error of zorro_util.py:862-863,
 * sum_i |cdf_i - (1 - 1/(1 + exp(-x1 (x0 - h_i)))^x2)|, over the box
 * [lo, hi].  The reference minimises it with unseeded basinhopping
 * (zorro.py:2008); this is a deterministic bounded Nelder-Mead (the
 * coefficients, start simplex and stopping tests of scipy's 'Nelder-Mead'
 * with bounds) from x0.  Host code; x_out[3], *f_out (may be null) and
 * *n_eval (may be null) receive the point, its value and the evaluations. */
int zr_logistic_fit(const double* h_sigma, const float* cdf, int nbins, const double* x0, const double* lo,
                    const double* hi, double xatol, double fatol, int maxiter, int maxfev, double* x_out,
                    double* f_out, int* n_eval);

/* ---- dose filter: doseFilter, zorro.py:2349-2494 ---- */

size_t zr_dose_work_bytes(int P0, int P1, int n_frames);
/* filt_sum [H][W] = |IFFT(sum_n FFT(pad_sym(aligned[n])) * thres_n * filt_n)|
 * cropped to H x W (np.pad 'symmetric' to P0 x P1).  aligned: [N][H][W] the
 * shifted frames (zr_shift_sum's ``aligned``); thres_q, dose_end: device
 * float arrays [N] (per-frame cut-off frequency thresQ and accumulated dose
 * at the end of the frame, zorro.py:2444-2452). */
int zr_dose_filter(const float* aligned, int N, int H, int W, const zr_dose_params_t* params,
                   const float* thres_q, const float* dose_end, int P0, int P1, float* filt_sum,
                   void* work, size_t work_bytes, void* stream);

/* ---- batches of movies: ImageRegistrator.alignImageStack over several
 * movies of one shape (zorro.py:773-1231 per movie) ----
 * A context holds the device buffers of the correlation stages for one shape
 * class (frame size, padded and cropped sizes, maxShift), sized by the limits
 * when it is created; zr_ctx_create is the one entry point here that
 * allocates.  zr_submit_batch queues, on ``stream``, the forward spectra of
 * every frame of every movie (xcorrnm2_tri, zorro.py:875-914), the frame
 * terms and the pair windows (mnxc2, zorro.py:1014-1097) and the peak search
 * (locatePeak, zorro.py:1099-1231) as one set of launches over all movies,
 * and returns.  zr_poll returns 1 when the batch has finished (0 while it
 * runs, a negative code on a CUDA error) and then has copied each movie's
 * records to its ``peaks`` (n_pairs records, in the order of its pairs);
 * zr_wait blocks until then.  One batch is in flight per context.  Every
 * record equals what the per-stage entry points give for that movie alone.
 * The drift solve and the later stages (zr_logistic_fit, zr_l1_solve,
 * zr_shift_sum, zr_dose_filter, zr_tiled_frc) follow per movie. */
typedef struct zr_ctx zr_ctx_t;
typedef struct zr_batch_limits {
  int height, width;      /* frame size (every movie of the class) */
  int P0, P1, C0, C1;     /* padded and Fourier-cropped sizes */
  int max_shift;          /* maxShift */
  int max_frames;         /* frames of all movies of one batch, at most */
  int max_pairs;          /* pairs of all movies of one batch, at most */
  int chunk_frames;       /* frames transformed per spectra launch */
} zr_batch_limits_t;
typedef struct zr_batch_movie {
  zr_frames_t frames;       /* the movie's frames (device); frame_movie NULL */
  const double* mean_sub;   /* [n_frames] subtracted before the transform (device; NULL: 0) */
  const int* pairs;         /* [n_pairs][2] (I, J), host memory, read during the call */
  int n_pairs;
  zr_peak_result_t* peaks;  /* [n_pairs] host memory, written by zr_poll / zr_wait */
} zr_batch_movie_t;
int zr_ctx_create(int device, const zr_batch_limits_t* limits, zr_ctx_t** ctx);
int zr_ctx_destroy(zr_ctx_t* ctx);
int zr_submit_batch(zr_ctx_t* ctx, const zr_batch_movie_t* movies, int n_movies, const zr_peak_params_t* params,
                    void* stream);
int zr_poll(zr_ctx_t* ctx);
int zr_wait(zr_ctx_t* ctx);

/* ---- compressed movie files: MRCZ (zorro.loadData, zorro.py:3414) ---- */

/* Decode one LZ4 block (blosc's LZ4 and LZ4HC codecs) of src_bytes into
 * dst (dst_bytes available).  Host memory, host code.  Returns the decoded
 * byte count, or -1 for a malformed block (nothing outside the buffers is
 * read or written). */
long long zr_lz4_decompress(const void* src, size_t src_bytes, void* dst, size_t dst_bytes);

/* ---- planning: FFTW_MEASURE and wisdom, pyFFTWPlanner zorro_util.py:966-1066 ---- */

/* A registration shape to plan for: padded size P0 x P1, Fourier crop
 * C0 x C1, maxShift, and the number of synthetic frames to measure on
 * (2..64; 8 is plenty). */
typedef struct zr_plan_shape {
  int P0, P1, C0, C1, max_shift, n_frames;
} zr_plan_shape_t;

/* Sequences per CTA (1, 2 or 4; 0 = the built-in default) of the forward
 * row pass (for transforms of P1 points), the forward column pass (P0), the
 * correlation column pass (C0) and the correlation row pass (C1), and the
 * measured milliseconds of every candidate: ms_spectra[rows][cols] and
 * ms_pairs[cols][rows] for the variants 1, 2, 4 in that order. */
typedef struct zr_plan_choice {
  int fwd_rows, fwd_cols, xc_cols, xc_rows;
  float ms_spectra[3][3];
  float ms_pairs[3][3];
} zr_plan_choice_t;

/* zr_plan measures, on the current device and ``stream``, the forward
 * spectra of n_frames synthetic P0 x P1 frames and the correlation windows
 * of all their pairs for every variant, keeps the fastest for this device
 * (for every later call with those transform lengths) and reports the
 * choice.  Blocking (it waits for its timings).  The variants split the
 * same transforms differently between CTAs: results do not depend on the
 * plan.  zr_plan_set installs a choice saved earlier (the caller's wisdom),
 * zr_plan_get reads the installed one (0 = default). */
size_t zr_plan_work_bytes(const zr_plan_shape_t* shape);
int zr_plan(const zr_plan_shape_t* shape, void* work, size_t work_bytes, void* stream, zr_plan_choice_t* out);
int zr_plan_set(const zr_plan_shape_t* shape, const zr_plan_choice_t* choice);
int zr_plan_get(const zr_plan_shape_t* shape, zr_plan_choice_t* choice);

#ifdef __cplusplus
}
#endif

#endif /* ZORRO_GB300_H */
