/*
 * libFourierConvolutionCUDA -- GB300 (sm_103a) drop-in for the native library behind
 * fiji/SPIM_Registration's multiview Bayesian deconvolution.
 *
 * Part 1 is the C ABI the reference binds through JNA (method name == symbol name); the
 * prototypes follow the Java interfaces they replace.  Part 2 adds status-returning and
 * whole-iteration entry points for a Java loop that keeps the views resident on the GPU.
 *
 * Conventions: all images are float32, x fastest (imglib2 ArrayImg layout).  The JNA calls
 * pass dimensions reversed, {z, y, x}, as MVDeconFFTThreads.getCUDACoordinates does
 * (spim/process/fusion/deconvolution/MVDeconFFTThreads.java:157-165); the mvd_* calls take
 * {x, y, z}.  Kernels have odd sizes with their centre at size/2.
 */
#ifndef MVDECON_H
#define MVDECON_H

#ifdef __cplusplus
extern "C" {
#endif

/* ===================== Part 1: the reference's JNA interface ===================== */

/* spim/process/cuda/CUDAStandardFunctions.java:36-44 */
int getCUDAcomputeCapabilityMinorVersion(int devCUDA);
int getCUDAcomputeCapabilityMajorVersion(int devCUDA);
/* -1 if the driver failed (CUDAStandardFunctions.java:38-41), else the device count */
int getNumDevicesCUDA(void);
/* writes a NUL-terminated name into a 256-byte buffer (CUDATools.java:76) */
void getNameDeviceCUDA(int devCUDA, char* name);
long long getMemDeviceCUDA(int devCUDA);
long long getFreeMemDeviceCUDA(int devCUDA);

/* spim/process/cuda/CUDAFourierConvolution.java:30 -- declared by the reference, never called
 * by it; returns NULL and records an error (mvd_last_error). */
float* convolution3DfftCUDA(float* im, int* imDim, float* kernel, int* kernelDim, int devCUDA);

/* spim/process/cuda/CUDAFourierConvolution.java:31, called from
 * MVDeconFFTThreads.java:86-89,109-112 and LRFFTThreads.java:70,85.
 * Convolves the block `im` (imDim = {z,y,x}) in place with `kernel` (kernelDim = {z,y,x},
 * odd sizes, centre at size/2): true convolution of the block extended mirror-single at its
 * border, the result the CPU FFTConvolution gives on the same block.  Callers consume the
 * interior [k/2, dim - k/2).  Synchronous; no pointer is kept.  On failure `im` is left
 * unmodified and the reason is available from mvd_last_error(). */
void convolution3DfftCUDAInPlace(float* im, int* imDim, float* kernel, int* kernelDim, int devCUDA);

/* ===================== Part 2: additions (status-returning) ===================== */

enum {
  MVD_OK = 0,
  MVD_ERR_ARG = 1,     /* invalid argument */
  MVD_ERR_CUDA = 2,    /* CUDA runtime error (see mvd_last_error) */
  MVD_ERR_NOMEM = 3,   /* device allocation failed */
  MVD_ERR_STATE = 4,   /* call not valid in the handle's state */
  MVD_ERR_INTERNAL = 5
};

/* PSFTYPE ordinals of spim/process/fusion/deconvolution/MVDeconFFT.java:49 */
enum {
  MVD_OPTIMIZATION_II = 0,
  MVD_OPTIMIZATION_I = 1,
  MVD_EFFICIENT_BAYESIAN = 2,
  MVD_INDEPENDENT = 3
};

/* handle flags */
enum {
  MVD_FLAG_PLAIN = 1,    /* reference structure: one block per launch sequence, separate
                            quotient / update kernels, no graph (the plain FP32 GPU form) */
  MVD_FLAG_NO_GRAPH = 2, /* batched, fused passes but launched eagerly (no CUDA graph) */
  MVD_FLAG_AUTOTUNE = 4, /* time candidate tile plans per view at creation and keep the fastest;
                            the choice is kept for the process, so later handles with the same
                            data-box and kernel sizes on the same device reuse it untimed */
  MVD_FLAG_TENSOR_DFT = 8 /* z passes of the compiled pencil lengths 320 and 288 run their middle
                             16-point DFTs on the tensor cores (TF32, three-term split, FP32
                             accumulation); other lengths stay on the FP32 SIMT path */
};

/* AdjustInput.sumImg's dependence on the thread count (AdjustInput.java:114-118): the Java code
 * adds the sum of portion 0 of FusionHelper.divideIntoPortions(n, 2 t) twice, so with t threads
 * each PSF and compound kernel is divided by its sum plus that portion's sum.  OR-ing
 * MVD_FLAG_REF_SUM_THREADS(t) (1 <= t <= 32767) into mvd_create's flags reproduces that
 * normalisation; without it every kernel is divided by its plain FP64 sum (unit sum). */
#define MVD_FLAG_REF_SUM_THREADS(t) ((int)((unsigned)(t) << 16))

/* Last error message of the calling thread ("" if none). */
const char* mvd_last_error(void);

/* Library version string. */
const char* mvd_version(void);

/* Status-returning convolution3DfftCUDAInPlace (same arguments and semantics). */
int mvd_convolve3d_inplace(float* im, const int* imDim, const float* kernel, const int* kernelDim,
                           int devCUDA);

/* Device-pointer convolution on `stream` (a cudaStream_t, NULL = the library's stream of
 * that device): out = ext(in) (*) kernel over dims_xyz.  ext_mode 0 = mirror-single,
 * 1 = constant ext_value.  in and out must not overlap.  Returns after enqueueing. */
int mvd_convolve3d_device(const float* in, float* out, const int* dims_xyz, const float* kernel,
                          const int* kdims_xyz, int ext_mode, float ext_value, int devCUDA,
                          void* stream);

/* No counterpart in the reference.  mvd_convolve3d_device without any device allocation, for
 * callers that may not call cudaMalloc / cudaFree while they run (a streaming acquisition
 * pipeline that cannot take an allocation's device-wide synchronisation, or a host framework
 * whose memory manager owns the device pool).  Same arguments and result as
 * mvd_convolve3d_device, with two differences: stream == NULL means the legacy default stream
 * (not the library's stream), and the call returns after enqueueing without waiting, so `out`
 * is ready only once that stream's work is done.  All working memory comes from one static
 * 64 MiB device array per GPU (held until the process exits), and sizes whose plans, spectra
 * and tables do not fit it are rejected with MVD_ERR_ARG and a message.  The first call on a
 * device looks the array up.  The call copies its small tables from host memory that is freed
 * on return, so it is refused (MVD_ERR_STATE) while `stream` is being captured.  Calls share
 * the array: calls that overlap on the GPU race and must be serialised by the caller. */
int mvd_convolve3d_device_noalloc(const float* in, float* out, const int* dims_xyz, const float* kernel,
                                  const int* kdims_xyz, int ext_mode, float ext_value, int devCUDA,
                                  void* stream);

/* ----- whole-deconvolution handle: MVDeconvolution / MVDeconInput / MVDeconFFT -----
 * (spim/process/fusion/deconvolution/MVDeconvolution.java:94-211, MVDeconFFT.java:79-324)
 * mvd_create uploads the views, weights and PSFs, prepares kernel1/kernel2 per PSFTYPE
 * (MVDeconFFT.init), their spectra and the tile plans, and initialises psi with the average
 * of the first iteration (MVDeconvolution.java:133-147).  Each view's convolutions cover only
 * the bounding box of its data (img > 0 or weight > 0), with all of its tiles, of whatever
 * shape, in one launch per pass.  block_xyz selects the reference's block size for
 * MVD_FLAG_PLAIN (NULL = one block of image + kernel - 1).  views, weights and psfs may point
 * to host memory or to device memory of devCUDA (copied on the handle's own stream: work that
 * writes them on another stream must be complete before the call). */
typedef struct mvd_decon mvd_decon;

int mvd_create(mvd_decon** out, int devCUDA, const int* dims_xyz, int num_views,
               const float* const* views, const float* const* weights, const float* const* psfs,
               const int* psf_dims_xyz /* 3 per view */, int psftype, double lambda, int flags,
               const int* block_xyz);
int mvd_destroy(mvd_decon* h);

/* One view stage: conv1 -> quotient -> conv2 -> update (MVDeconvolution.java:374-462). */
int mvd_run_view(mvd_decon* h, int view);
/* One iteration = every view in order (MVDeconvolution.runIteration, :349-465). */
int mvd_run_iteration(mvd_decon* h);
/* `iterations` iterations back to back. */
int mvd_run(mvd_decon* h, int iterations);
/* Wait for queued work. */
int mvd_synchronize(mvd_decon* h);

/* psi in/out (x fastest, N floats).  mvd_get_psi with masked != 0 applies the reference's
 * final masking (psi = 0 where no view has data, MVDeconvolution.java:201-208) to the copy. */
int mvd_get_psi(mvd_decon* h, float* psi, int masked);
int mvd_set_psi(mvd_decon* h, const float* psi);
/* psi value set by the first iteration (FP64 average). */
int mvd_get_initial_average(mvd_decon* h, double* avg);
/* kernel2 of a view (the compound / mirrored kernel), psf-sized. */
int mvd_get_kernel(mvd_decon* h, int view, int which /* 1 or 2 */, float* out);

/* Per-view statistics of an iteration ("sum change", "max change per pixel",
 * MVDeconvolution.java:447-457); `iteration` counts from 0, the last 64 are kept. */
int mvd_get_stats(mvd_decon* h, int iteration, int view, double* sum_change, double* max_change);
int mvd_get_iteration(mvd_decon* h, int* iteration);

/* Tile plan of a view: tiles per axis, tile size, effective size, padded voxels. */
int mvd_get_plan(mvd_decon* h, int view, int* tiles_xyz, int* tile_xyz, int* eff_xyz,
                 long long* padded_voxels);

/* The kernels the view's plan runs (chosen by MVD_FLAG_AUTOTUNE, else the defaults): *threads =
 * the plane kernels' CTA size; *variant bit 0 = compile-time-shaped kernels, bit 1 = radices in
 * ascending order (generic kernels), bit 2 = tensor-core middle DFT stage in the z pass, bit 3 =
 * in-place plane kernels staged through tensor memory (two CTAs per SM).  No counterpart in the
 * reference. */
int mvd_get_plan_variant(mvd_decon* h, int view, int* threads, int* variant);

/* The cudaStream_t the handle enqueues on (for events recorded by the caller). */
int mvd_get_stream(mvd_decon* h, void** stream);

/* Kernel launches the handle has issued so far (graph replays count every node). */
int mvd_get_launch_count(mvd_decon* h, long long* launches);

/* Runs one iteration eagerly with CUDA events around each pass and returns the summed
 * device time per pass kind in milliseconds: ms[0] forward plane passes, ms[1] z passes,
 * ms[2] inverse plane + quotient, ms[3] inverse plane + update (whose last CTA also files the
 * view's statistics), ms[4] everything else (nothing in the fused form); launches[k] the number
 * of launches of each kind. */
int mvd_profile_iteration(mvd_decon* h, double* ms, int* launches);

/* ----- forward / backward of the multiview Poisson image-formation model -----
 * No counterpart in the reference (its Java code has no gradients); the pair that PSF
 * refinement from bead data needs, the analogue of a torch.autograd.Function:
 *   f_v = ext(psi) (*) kernel1_v        (mirror-single extension, as in the first convolution)
 *   NLL = sum_v sum_{x: img_v > 0} w_v (f_v - img_v log f_v)
 * mvd_forward returns NLL (FP64 sum).  mvd_backward writes dNLL/dpsi (N floats) and
 * dNLL/dkernel1_v (psf-sized, one buffer per view); each view's blur is recomputed tile by
 * tile instead of being kept.  Fused handles only (not MVD_FLAG_PLAIN). */
int mvd_forward(mvd_decon* h, double* nll);
int mvd_backward(mvd_decon* h, float* grad_psi, float* const* grad_psf);
/* Replace kernel1 (the PSF used by the first convolution and the model) or kernel2 of a view,
 * as given (no normalisation), and its spectra -- e.g. after a projected gradient step. */
int mvd_set_kernel(mvd_decon* h, int view, int which /* 1 or 2 */, const float* data);

/* ----- input preparation (the views in the fused frame and their weights), on the GPU -----
 * TransformInput.loop (spim/process/fusion/deconvolution/TransformInput.java:90-116) and
 * TransformWeights with BlendingRealRandomAccess.computeWeight
 * (spim/process/fusion/weights/BlendingRealRandomAccess.java:91-121).  For every voxel
 * (x, y, z) of the fused output box (dims out_dims_xyz, global position + offset_xyz) the view
 * position is t = affine^-1 (position), `affine` being the view's row-packed 3x4 registration
 * (view -> world, imglib2 AffineTransform3D order).  out_img (may be NULL): trilinear value of
 * the view extended mirror-single, clamped to >= 1e-4 where t lies inside the view, else 0
 * ("no data").  out_blend (may be NULL): the cosine blending weight at t over the view's
 * interval with border_xyz / blending_xyz.  Device pointers; enqueued on `stream`. */
int mvd_transform_view(const float* view, const int* view_dims_xyz, const double* affine, const int* offset_xyz,
                       const int* out_dims_xyz, float* out_img, float* out_blend, const float* border_xyz,
                       const float* blending_xyz, int devCUDA, void* stream);
/* WeightNormalizer's normalisation with the OSEM factor, in place on `num_views` device weight
 * volumes of n voxels (WeightNormalizer.java:73-253, ProcessForDeconvolution.java:372-405).
 * mode 0, VIRTUAL (NormalizingRandomAccess.java:57-66): w_v / (sum_w > 1 ? sum_w : 1), then
 * min(1, w * osem).  mode 1, PRECOMPUTED (WeightNormalizer.ApplyDirectly): w_v / sum_w, then
 * min(1, w * (float)osem); NaN where no view has weight, as in the reference.  Results equal
 * the reference's double arithmetic bit for bit (certified float-pair arithmetic, with the rare
 * undecided voxels finished in double).  Allocates a stream-ordered scratch list. */
int mvd_normalize_weights(float* const* weights, int num_views, long long n, double osem, int mode, int devCUDA,
                          void* stream);
/* WeightNormalizer's overlap statistics (WeightNormalizer.java:94-106, 187-252), which
 * ProcessForDeconvolution uses as the automatic OSEM factor (:352-356): the minimum over all
 * voxels of the number of views with weight > 0, and the mean over the num_portions portions
 * of FusionHelper.divideIntoPortions(n, num_portions) of each portion's mean count (the
 * reference uses 2 x its thread count).  Run on the weights before normalisation (a weight's
 * sign does not change); waits for `stream`. */
int mvd_weight_overlap(const float* const* weights, int num_views, long long n, int num_portions, int* min_views,
                       double* avg_views, int devCUDA, void* stream);

/* ----- PSF pipeline (spim/process/fusion/deconvolution/ExtractPSF.java), on the GPU -----
 * mvd_extract_psf: ExtractPSF.extractPSFLocal (:374-415): psf[p] = sum over the bead
 * locations (x, y, z triples, doubles, in the view's pixel frame; host array) of the view
 * (device, dims_xyz) interpolated trilinearly, extended periodically, at p - psf_dims / 2 +
 * location; locations are added in the given order.  normalize != 0 then applies
 * ExtractPSF.normalize (:298-316): (v - min) / (max - min).  psf: device, overwritten. */
int mvd_extract_psf(const float* img, const int* dims_xyz, const double* locations_xyz, int num_locations,
                    const int* psf_dims_xyz, float* psf, int normalize, int devCUDA, void* stream);
/* ExtractPSF.transformPSF (:325-372), host only: the odd size of the transformed PSF (the
 * bounding box of model applied to [0, dim - 1], (int)extent + 1, made odd) and the offset that
 * maps the PSF's centre voxel (dim / 2) to the centre of the result. */
int mvd_transformed_psf_size(const int* psf_dims_xyz, const double* model, int* out_dims_xyz, double* offset_xyz);
/* ExtractPSF.transform (:417-464): out[p] = psf(model^-1 (p + offset)), trilinear over the PSF
 * extended with zeros.  `model` is the view's row-packed 3x4 registration; device buffers. */
int mvd_transform_psf(const float* psf, const int* psf_dims_xyz, const double* model, const int* out_dims_xyz,
                      const double* offset_xyz, float* out, int devCUDA, void* stream);

/* ----- separable convolution (the difference-of-Gaussian detector's native library) -----
 * The JNA interface spim/process/cuda/CUDASeparableConvolution.java:34-46 (loaded from a file
 * whose name contains "separable": the alias libSeparableConvolutionCUDALib.so of this
 * library).  convolve_K convolves `image` (imageW x imageH x imageD floats, x fastest) in place
 * along x, then y, then z, each axis only when its flag is set, with K-tap kernels (the
 * caller centres shorter kernels in zeros, CUDASeparableConvolutionFunctions.java:253-265):
 * out[x] = sum_{j=-R..R} in[x + j] k[R - j], R = K / 2, accumulated in float in order of j.
 * Each pass extends its own input: outofbounds 0 = zero, 1 = outofboundsvalue, 2 = the border
 * pixel.  Returns nonzero on success (JNA boolean); on failure the image is unchanged and the
 * reason goes to stderr and mvd_last_error().  devCUDA = -1 (the reference's CPU request)
 * runs on GPU 0. */
int convolve_127(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                 int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA);
int convolve_63(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA);
int convolve_31(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA);
int convolve_15(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
                int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA);
int convolve_7(float* image, float* kernelX, float* kernelY, float* kernelZ, int imageW, int imageH, int imageD,
               int convolveX, int convolveY, int convolveZ, int outofbounds, float outofboundsvalue, int devCUDA);
/* CUDASeparableConvolution.convolutionCPU (:44): all three axes with kernels of 2 r + 1 taps
 * (r <= 63).  This library has no CPU code path: it computes on GPU 0. */
void convolutionCPU(float* image, float* kernelX, float* kernelY, float* kernelZ, int kernelRX, int kernelRY,
                    int kernelRZ, int imageW, int imageH, int imageD, int outofbounds, float outofboundsvalue);
/* The same passes on device memory (no counterpart in the reference): `image` and `scratch`
 * are device buffers of dims_xyz floats; kernels[a] (host, taps[a] odd <= 127 values, NULL =
 * skip axis a).  *result receives the buffer that holds the output (image or scratch).
 * Enqueued on `stream`. */
int mvd_separable_convolve_device(float* image, float* scratch, const float* const* kernels, const int* taps,
                                  const int* dims_xyz, int outofbounds, float outofboundsvalue, int devCUDA,
                                  void* stream, float** result);

#ifdef __cplusplus
}
#endif

#endif /* MVDECON_H */
