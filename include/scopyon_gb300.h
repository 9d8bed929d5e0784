/*
 * scopyon_gb300 — C ABI of the GB300 image-formation engine.
 *
 * Every function takes device pointers (memory the caller allocated on the
 * current CUDA device), sizes, a host pointer to a parameter struct where
 * needed, and a cudaStream_t passed as void*.  Functions only enqueue work on
 * that stream; they never allocate device memory and never synchronise except
 * where stated.  Return value: 0 on success, a negative SC_ERR_* code
 * otherwise; sc_last_error() gives a message (thread-local).
 *
 * Reference citations are paths inside the ecell/scopyon source tree.
 */
#ifndef SCOPYON_GB300_H
#define SCOPYON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SC_OK 0
#define SC_ERR_ARG (-1)      /* invalid argument (host-side validation)      */
#define SC_ERR_CUDA (-2)     /* a CUDA call or launch failed                  */
#define SC_ERR_TIMEOUT (-3)  /* a bounded device-side wait ran out            */
#define SC_ERR_NAN (-4)      /* non-finite input detected                     */
#define SC_ERR_CAPACITY (-5) /* a caller buffer is too small                  */

#define SC_PSF_BORN_WOLF 0
#define SC_PSF_GAUSSIAN 1

#define SC_CAM_EMCCD 0
#define SC_CAM_CCD 1
#define SC_CAM_CMOS_TABLE 2
#define SC_CAM_SCMOS 3

/* Status word written by kernels into a caller buffer (int[4]):
 * [0] error flags (bit0 bad PSF key, bit1 missing table, bit2 bounds overflow,
 *     bit3 RNG loop bound hit, bit4 capacity, bit5 a bounded wait for an
 *     asynchronous copy ran out, bit6 a caller-built record with a negative
 *     first pixel, which is not binned, bit7 a non-finite emitter position or
 *     normalisation, bit8 an index out of range in a library built with
 *     -DSC_BOUNDS_CHECK: [1] the index, [2] its bound, [3] the check's site),
 *     [1..3] first offending index. */
#define SC_STATUS_WORDS 4

/* One emitter during one exposure sub-step, ready to be splatted (64 bytes).
 * The first 32 bytes are all the box path reads. */
typedef struct {
    int64_t box_off;     /* box path: float index of pixel (i_start, j_start)'s entry */
    int16_t i_start, n_i;/* first pixel index and number of footprint bounds along x  */
    int16_t j_start, n_j;/* same along y; n_i < 2 or n_j < 2 means nothing to splat   */
    float w;             /* normalisation * res^2: photons per unit table sum          */
    int32_t slot;        /* PSF table slot of the depth key; -1: nothing to splat      */
    int32_t box;         /* 0: summed-area path; else bounds are l0 + P*k exactly and  */
                         /* box - 1 is the phase (m_x mod P) * P + (m_y mod P) of the   */
                         /* box-table block that holds the footprint                   */
    int32_t box_local;   /* box path: that entry's (row << 16) | column in its block   */
    double x0, y0;       /* footprint origin along x / y in metres (exact FP64)      */
    float ax_hi, ax_lo;  /* (i_start*px - x0)/res as a double-float                   */
    float ay_hi, ay_lo;  /* (j_start*px - y0)/res as a double-float                   */
} ScStepRec;

typedef struct {
    /* optics and geometry */
    double px;               /* pixel length on the sample: pixel_length / magnification */
    double res;              /* PSF grid resolution (1 nm)                                */
    double depth_cutoff;     /* fluorophore.depth_cutoff                                  */
    double focal[3];         /* detector.focal_point                                      */
    int32_t nw, nh;          /* image size (pixels along x, y)                            */
    int32_t n_signal;        /* cartesian PSF grid edge, 2 * n_r - 1                       */
    int32_t n_sub;           /* sub-steps in this frame                                   */
    int32_t n_particles;     /* particles per sub-step                                    */
    int32_t max_key;         /* largest valid depth key; key -1 maps to slot max_key + 1   */
    /* emission physics (reference _epifm.py:1267-1360) */
    double amplitude0;       /* Snell's-law amplitude, photons / s / m^2                   */
    double penetration;      /* evanescent penetration depth (inf for EPI)                */
    double x_sec;            /* absorption cross-section ln(10) * eps * 0.1 / N_A, m^2     */
    double qy;               /* quantum yield                                              */
    double beer;             /* 1 - 10^-A, fraction absorbed (Beer-Lambert)                */
    double norm_coeff;       /* sum(fluoem_norm) * psf_normalization                       */
    int32_t bleaching;       /* 1: photon-budget bleaching on                              */
    int32_t with_optinfo;    /* 1: accumulate the 8-vector true_data per particle          */
    int32_t box_p;           /* px / res when it is an integer P (box tables built), else 0 */
    int32_t box_nq;          /* pixel offsets per box-table axis, (n_signal+P-1)/P + 1      */
    int32_t row_layout;      /* sc_emitter_steps input rows: 0 [depth, x, y, m_id, p_state] */
                             /* FP64; 1 [depth, x, y, 0] FP32 with m_id the slot and       */
                             /* p_state 1 (sc_diffuse_steps layout 1)                       */
    int32_t pad;
} ScStepParams;

typedef struct {
    int32_t nw, nh;          /* image size                                                 */
    int32_t tile;            /* tile edge in pixels (8, 16 or 32)                          */
    int32_t halo;            /* pixels a footprint reaches past its first: ceil(sw/px) + 1 */
    int32_t warps;           /* warps per tile CTA (4 or 8)                                */
    int32_t tiles_x, tiles_y;
    int32_t n_r;             /* radial samples; quadrant table is (n_r+1)^2               */
    int32_t sat_pitch;       /* row pitch of one quadrant table in float2 entries          */
    int32_t n_images;        /* frames/images splatted by one launch                        */
    int32_t rec_per_image;   /* records per image (record r is in image r / rec_per_image); */
                             /* 0 means every record belongs to image 0                     */
    int32_t box_p, box_nq;   /* box tables: P rows per pixel and NQ pixel offsets, or 0     */
    int32_t n_slots;         /* depth-key tables held in d_sat / d_box                      */
    int32_t box_stages;      /* block copies in flight per splat warp (1..8; 0: 4)          */
    int32_t first_wait_polls;/* test hook: polls allowed for each splat warp's first block  */
                             /* wait; 0: the normal bound (4096), -1: none, so that wait    */
                             /* runs out at once (status bit 5) while the copies in flight  */
                             /* are still drained under the normal bound                   */
    int32_t box_kernel;      /* box path: 0 block copies into a shared-memory ring per warp */
                             /* (cp.async.bulk + mbarrier), 1 16-byte loads into registers  */
    int32_t pad;
    double px, res;
} ScSplatParams;

typedef struct {
    int32_t nw, nh;
    int32_t camera;          /* SC_CAM_*                                                   */
    int32_t exact;           /* 1: FP64 ADC arithmetic identical to the reference           */
    int32_t rounding;        /* 1: rint the ADC output                                     */
    int32_t bit;
    double qe, background, readout_noise, emgain, fullwell;
    double offset0, gain0;   /* used when the offset / gain maps are NULL                   */
    int32_t table_n;         /* CMOS noise table length                                    */
    uint64_t seed;           /* Philox key for native draws                                */
    uint64_t counter;        /* Philox counter base (e.g. frame index)                     */
    const int64_t *d_frame;  /* optional device counter f added to counter (graph replay)   */
    const double *d_photons64; /* exact mode: FP64 photons read in place of d_photons       */
    double *d_expect64;      /* exact mode: FP64 expectation QE*(photons+background) out    */
    const void *d_poisson_table; /* native mode: the tables of sc_poisson_table (required)   */
} ScCameraParams;

typedef struct {
    int32_t n_particles, n_sub;
    int32_t ndim;            /* 2: (x, y) inputs, depth 0; 3: (x, y, z)                    */
    int32_t boundary;        /* 0 none (reference), 1 periodic, 2 reflecting               */
    int32_t n_class;         /* diffusion classes in d_sigma                                */
    int32_t layout;          /* sc_diffuse_steps rows: 0 [depth, x, y, id, 1] FP64 (40 B);  */
                             /* 1 [depth, x, y, 0] FP32 (16 B; native draws and the        */
                             /* identity transform only)                                   */
    int64_t step0;           /* global index of the frame's first sub-step (Philox counter) */
    uint64_t seed;           /* Philox key                                                  */
    const int64_t *d_frame;  /* optional device counter f: step0 += f * n_sub (graph replay) */
    double lower[3], upper[3];        /* box of the periodic / reflecting boundary          */
    double scale, origin[3], unit_x[3], unit_y[3], unit_z[3];  /* preprocessing transform  */
    const double *d_class_box;        /* optional [n_class][6] (lower xyz, upper xyz): a box */
                                      /* per diffusion class in place of lower / upper       */
    const double *d_trans;            /* optional [n_sub][n_class][n_class] cumulative       */
                                      /* transition probabilities per sub-step: after its    */
                                      /* move, a particle in class a goes to the first b with*/
                                      /* d_trans[s][a][b] >= u (sampling2.py:52-68); the     */
                                      /* class array is then updated in place                */
    const double *d_uniforms;         /* optional [n_sub][n_particles] u for d_trans in place*/
                                      /* of Philox (the reference's draws)                   */
} ScDiffuseParams;

int sc_get_version(void);

/* sizeof of the ABI structs as this library was compiled: out[0..5] =
 * ScStepRec, ScStepParams, ScSplatParams, ScCameraParams, ScDiffuseParams,
 * ScGaussParams (n >= 6), so that a binding can check its layouts.          */
int sc_struct_sizes(size_t *out, int n);

/* *d_counter += delta on the stream: advances the device frame counter read by
 * sc_diffuse_steps and sc_camera, so that a captured frame can be replayed. */
int sc_counter_add(int64_t *d_counter, int64_t delta, void *stream);
const char *sc_last_error(void);

/* Host helper of the frame upload (no device work): one pass over a
 * sub-step's n rows [depth, x, y, id, state] (row-major FP64) that checks
 * each id against ids[i] (the known slot order), copies the rows to dst (the
 * pinned staging buffer) and writes the depth range to depth_range[0..1]
 * (NaN when a depth is NaN).  Returns 1 at the first differing id (the
 * caller then takes the general path), 0 otherwise.  Replaces the per-frame
 * stacking of EPIFMSimulator.__format_data's output
 * (src/scopyon/base.py:61-110) and the depth scan of
 * _EPIFMSimulator.output_frame (src/scopyon/_epifm.py:1121-1225).          */
int sc_stage_rows(const double *src, int64_t n, const double *ids, double *dst,
                  double *depth_range);

/* Radial PSF tables for n_keys depths, n_r radii each (r_i = i * res).
 * Replaces PointSpreadingFunction.get_born_wolf_distribution /
 * get_gaussian_distribution (src/scopyon/_epifm.py:136-213).               */
int sc_psf_radial(int kind, double wavelength, double na, double sigma,
                  const double *d_depths, int n_keys, int n_r, double res,
                  double *d_radial, void *stream);

/* Quadrant summed-area tables (double-float pairs) of the cartesian PSF grid,
 * one per radial table.  Replaces PointSpreadingFunction.radial_to_cartesian
 * (src/scopyon/_epifm.py:99-126) and the per-pixel slice sums of
 * overlay_signal_ (src/scopyon/_epifm.py:277-282).                          */
int sc_psf_quadrant_sat(const double *d_radial, int n_keys, int n_r, double res,
                        float *d_sat, int sat_pitch, void *stream);

/* Brownian sub-steps of one frame on the device.  d_pos (n x 3, sampling
 * frame, updated in place) holds the positions at the frame's first time
 * point; for each sub-step the formatted position [depth, x, y, id, 1] goes to
 * d_particles ([n_sub][n][5], the layout sc_emitter_steps reads; with
 * p->layout 1, [n_sub][n] rows [depth, x, y, 0] of FP32; d_particles NULL: no
 * rows) and the particle then moves by sigma * N(0, 1) per axis, with d_sigma
 * [n_sub][n_class][3] (sqrt(2 D dt) per step, class and axis) and d_class
 * (n, NULL = class 0).  Normals from d_normals ([n_sub][n][ndim]) when given,
 * with FP64 moves (the reference's arithmetic); else from Philox, with the
 * positions rounded to FP32 on entry and moved in FP32.  With p->d_trans, each particle's class
 * changes after every move as the transition table says and d_class (then
 * required) is updated in place.  Replaces move_points / sample_inputs
 * (src/scopyon/sampling.py:88-162) and sampling2.__move_points /
 * __transition_states (src/scopyon/sampling2.py:33-68).                    */
int sc_diffuse_steps(const ScDiffuseParams *p, double *d_pos, int32_t *d_class,
                     const double *d_sigma, const double *d_normals, double *d_particles,
                     void *stream);

/* Box-integrated PSF tables for an integer pixel pitch of P grid rows: for
 * every pixel start row m_x, m_y in [-P, NQ*P - P), the sum of the cartesian
 * grid over [m_x, m_x+P) x [m_y, m_y+P) clipped to the grid, stored as FP32 in
 * phase-major order [key][m_x mod P][m_y mod P][m_x div P][m_y div P] (with m
 * shifted by +P), NQ = (2 n_r - 1 + P - 1) / P + 1.  Each (m_x mod P,
 * m_y mod P) phase block of NQ x NQ values starts SC_BOX_BLOCK_FLOATS(NQ)
 * floats after the previous one (NQ^2 rounded up to SC_BOX_ALIGN_FLOATS
 * floats, 16 bytes by default, padding zero),
 * so a key takes P * P * SC_BOX_BLOCK_FLOATS(NQ) floats.  Built from the
 * quadrant tables of sc_psf_quadrant_sat.  With it, one emitter's footprint
 * is one contiguous, 16-byte aligned block (the pixel sums of
 * overlay_signal_, src/scopyon/_epifm.py:277-282).                         */
#ifndef SC_BOX_ALIGN_FLOATS
#define SC_BOX_ALIGN_FLOATS 4
#endif
#define SC_BOX_BLOCK_FLOATS(nq) \
    ((((nq) * (nq)) + SC_BOX_ALIGN_FLOATS - 1) & ~(SC_BOX_ALIGN_FLOATS - 1))

/* SC_BOX_BLOCK_FLOATS(nq) as this library was built (floats from one phase
 * block's start to the next).                                             */
int sc_box_block_floats(int nq);

/* Sets the largest L2 fetch from DRAM (32, 64 or 128 bytes; 0 the driver's
 * choice) as a hint for the current device's context in this process
 * (cudaLimitMaxL2FetchGranularity): the splat's random 784-byte box-table
 * blocks and 32-byte record heads then move about 842 bytes per record
 * instead of about 1,010.  It applies to every kernel of the process until
 * the process ends or the next call, and changes no setting of the GPU
 * itself.  No counterpart in the reference (a CPU program).                */
int sc_set_l2_fetch_granularity(int bytes);

/* Copies `bytes` from src to dst on `stream` (one cudaMemcpyAsync; the
 * direction follows from the addresses).  For a host without a device
 * runtime of its own: a frame's rows to the device before sc_emitter_steps,
 * its ADC counts and status words back after the camera.  From pinned host
 * memory the copy is asynchronous; from pageable memory it returns once the
 * source has been read.  No counterpart in the reference (a CPU program).  */
int sc_copy_async(void *dst, const void *src, size_t bytes, void *stream);

int sc_psf_box_table(const float *d_sat, int n_keys, int n_r, int sat_pitch, int box_p,
                     float *d_box, void *stream);

/* Emitter physics for one frame: excitation, emitted photons, photon-budget
 * bleaching, normalisation, depth key and footprint origin per particle and
 * sub-step.  d_particles is [n_sub][n_particles][5] (depth, x, y, m_id,
 * p_state) as formatted by EPIFMSimulator.__format_data, or with
 * p->row_layout 1 the FP32 rows [n_sub][n_particles][4] of sc_diffuse_steps
 * (layout 1) at the same address; d_present
 * ([n_sub][n_particles] bytes, NULL = all present) marks particle slots
 * absent at a sub-step; d_budget holds the
 * photon budget per particle slot (initialised by the caller at first sight,
 * carried across frames); d_optinfo receives the per-slot 8-vector sums of
 * the frame (may be NULL when with_optinfo is 0); d_norm, when not NULL,
 * receives each record's FP64 normalisation ([n_sub][n_particles]; 0: nothing
 * to splat), which sc_splat_fp64 reads.  Replaces
 * _EPIFMSimulator.__overlay_molecule_plane and get_emit_photons
 * (src/scopyon/_epifm.py:1267-1360).                                       */
int sc_emitter_steps(const ScStepParams *p, const double *d_particles,
                     const double *d_unit_time, const uint8_t *d_present,
                     const int32_t *d_key_slot,
                     double *d_budget, double *d_optinfo, ScStepRec *d_recs,
                     double *d_norm, int32_t *d_status, void *stream);

/* Native frame records: sc_diffuse_steps and sc_emitter_steps in one pass
 * for trajectories that live on the device.  For every (sub-step, particle)
 * the Brownian move, excitation, emitted photons, photon budget, depth key
 * and footprint are computed in the same order and with the same operations
 * as those two calls, so d_recs ([n_sub][n_particles]) equals theirs bit for
 * bit; the formatted positions are not stored.  d_pos and d_budget are
 * advanced to the end of the frame.  With bin_p (else NULL), each record is
 * also counted into its tile bin in d_bin_ws (a full sc_bin_workspace_bytes
 * workspace whose counts sc_bin_reset cleared), ready for sc_bin_finish.  Replaces move_points and
 * __overlay_molecule_plane (src/scopyon/sampling.py:88-119,
 * src/scopyon/_epifm.py:1267-1360).                                        */
int sc_native_records(const ScDiffuseParams *p, const ScStepParams *sp, double *d_pos,
                      int32_t *d_class, const double *d_sigma, const double *d_normals,
                      const double *d_unit_time, double *d_budget, const int32_t *d_key_slot,
                      ScStepRec *d_recs, const ScSplatParams *bin_p, void *d_bin_ws,
                      size_t bin_ws_bytes, int32_t *d_status, void *stream);

/* Bytes of scratch sc_bin_steps uses for n_rec records on n_tiles_total
 * tiles: the counts and cursors of every bin (16 bytes per tile), the bin and
 * rank of every record (8 bytes each), and a list of the bins too long to
 * sort in one warp (8 bytes per tile + 4).  A workspace of only the first
 * part is also accepted; the scatter then recomputes each record's bin and
 * long bins are sorted by one warp each.                                    */
size_t sc_bin_workspace_bytes(int n_rec, int n_tiles_total);

/* Clears the bin counts of a binning workspace (a memset on the stream). */
int sc_bin_reset(const ScSplatParams *p, void *d_ws, size_t ws_bytes, void *stream);

/* Scan, placement and per-bin sort of records a producer has counted into a
 * full binning workspace (sc_native_records with bin_p): the second half of
 * sc_bin_steps, with the same outputs.                                      */
int sc_bin_finish(int n_rec, const ScSplatParams *p, void *d_ws, size_t ws_bytes,
                  int32_t *d_tile_start, int32_t *d_items, void *stream);

/* Deterministic counting sort of records by the tile that holds their first
 * footprint pixel, box-path records in bins [0, n_tiles) and summed-area-path
 * records in bins [n_tiles, 2 n_tiles); d_items receives the record indices
 * grouped by bin (ascending within a bin), d_tile_start (2 n_tiles + 1) the
 * bin offsets.  (New: the reference adds particle by particle,
 * src/scopyon/_epifm.py:1262-1264.)                                        */
int sc_bin_steps(const ScStepRec *d_recs, int n_rec,
                 const ScSplatParams *p, void *d_ws, size_t ws_bytes,
                 int32_t *d_tile_start, int32_t *d_items, int32_t *d_status, void *stream);

/* ---------------------------------------------------------------------------
 * Differentiable expected image (Gaussian PSF).  The reference's Gaussian
 * point-spread function (src/scopyon/_epifm.py:133-134), integrated over each
 * pixel analytically instead of on its 1-nm grid (:224-282), with the TIRF
 * excitation exp(-|z - z_focal| / d) of :1281-1289 as depth dependence:
 *   mu[f][i][j] = bg[f] + sum_e I_e A(z_e) Gx_e(i) Gy_e(j).
 * Emitters are float4 (x, y, z, I): metres from the image centre and photons;
 * sigma (metres) is a device scalar.  New in this engine: the reference has
 * no gradients.                                                              */
typedef struct {
    int32_t nw, nh;          /* image size                                        */
    int32_t n_frames;        /* frames, each with n_emit emitters                 */
    int32_t n_emit;
    int32_t half_win;        /* R: a (2R+1)^2 pixel window per emitter (1..15)    */
    int32_t tile;            /* forward tile edge (8 or 16)                       */
    double px;               /* pixel length on the sample (metres)               */
    double inv_pen;          /* 1 / penetration depth (0: EPI, A = 1)             */
    double z_focal;
} ScGaussParams;

/* Bytes of device workspace sc_gauss_forward needs. */
size_t sc_gauss_workspace_bytes(const ScGaussParams *p);

/* d_mu[n_frames][nw][nh] = expected photons (d_bg[n_frames] may be NULL). */
int sc_gauss_forward(const ScGaussParams *p, const float *d_emit, const float *d_sigma,
                     const float *d_bg, void *d_ws, size_t ws_bytes, float *d_mu,
                     int32_t *d_status, void *stream);

/* Adjoint of sc_gauss_forward: from d_grad_mu = dL/dmu, d_grad_emit (float4
 * per emitter: dL/dx, dL/dy, dL/dz, dL/dI) and, if not NULL, each emitter's
 * share of dL/dsigma (sum them for the total; dL/dbg[f] is the sum of
 * d_grad_mu over frame f).  d_ws is the workspace sc_gauss_forward filled for
 * the same p, emitters and sigma (its records and tile bins are reused); it
 * must not have been reused in between.                                     */
int sc_gauss_backward(const ScGaussParams *p, const float *d_emit, const float *d_sigma,
                      const void *d_ws, size_t ws_bytes, const float *d_grad_mu,
                      float *d_grad_emit, float *d_grad_sigma_e, void *stream);

/* Spot fits for n_blobs blobs (d_blobs: [n][3] x, y, r in pixels) in a
 * double image [nw][nh]: the region of +-roi_size pixels around each blob,
 * a least-squares plane through its four edges, and a 2-D Gaussian
 * a1 exp(-((x - a2)^2 + (y - a3)^2) / a4) fitted to the remainder from the
 * reference's start.  d_out[n][8] = (centre x, centre y, intensity,
 * background, a1, a4, status, 0); status 0 is a spot, 1 a region summing to
 * <= 0, 2 a failed fit, 3 a centre outside the region.  Replaces
 * spot_detection with given blobs (src/scopyon/analysis/spot_detection.py:49-173). */
int sc_spot_fit(const double *d_image, int nw, int nh, const double *d_blobs, int n_blobs,
                double roi_size, double *d_out, void *stream);

/* Bytes of scratch the two reductions below need for n_seg segments of
 * seg_len values (partial sums of up to 64 CTAs per segment).               */
size_t sc_reduce_scratch_bytes(int64_t seg_len, int n_seg);

/* d_out[s] = sum of d_x[s * seg_len .. (s + 1) * seg_len) in FP64, in a fixed
 * order (deterministic). */
int sc_segment_sum(const float *d_x, int64_t seg_len, int n_seg, void *d_scratch,
                   size_t scratch_bytes, double *d_out, void *stream);

/* Poisson negative log-likelihood per segment, sum(mu - k log mu) accumulated
 * in FP64, and (if d_grad_mu is not NULL) its gradient 1 - k / mu.           */
int sc_poisson_nll(const float *d_mu, const float *d_counts, int64_t seg_len, int n_seg,
                   void *d_scratch, size_t scratch_bytes, double *d_loss, float *d_grad_mu,
                   void *stream);

/* ---------------------------------------------------------------------------
 * Gradient through diffusion (new: the reference has no gradients).  Emitter
 * e (float4 x, y, z, I) moves in 2-D as p_t = p0 + sqrt(2 D dt) Z_t, Z_t the
 * sum of its first t Philox normal pairs (src/scopyon/sampling.py:88-119),
 * and contributes I / T photons at each of T sub-steps (the unit_time
 * weights of src/scopyon/_epifm.py:1183-1199).  D is a device scalar (m^2/s).
 * Positions are regenerated from the counters, never stored across passes.  */

/* Bytes of scratch sc_gauss_nll / sc_diffusion_dD need for n values. */
size_t sc_dgrad_scratch_bytes(int64_t n_values);

/* d_out[t][e] = (x_t, y_t, z, I / T), t < T.  d_normals ([T][n][2], else
 * NULL) replace the Philox draws.                                          */
int sc_diffusion_positions(const float *d_emit, int n, int T, const float *d_D, double dt,
                           uint64_t seed, const float *d_normals, float *d_out, void *stream);

/* Gaussian approximation of the camera likelihood of counts k given mu, with
 * variance mu + r2 (r2: d_var_map per pixel, else var):
 * *d_loss = sum (k - mu)^2 / (2 v) + log(v) / 2 (FP64), d_grad_mu = dL/dmu.  */
int sc_gauss_nll(const float *d_mu, const float *d_counts, int64_t n, const float *d_var_map,
                 double var, void *d_scratch, size_t scratch_bytes, double *d_loss,
                 float *d_grad_mu, void *stream);

/* *d_dD = sum_{t,e} dL/dp_t . (p_t - p0) / (2 D) (FP64) from the positions of
 * sc_diffusion_positions and their gradients (float4: dL/dx, dL/dy, ...).   */
int sc_diffusion_dD(const float *d_pos, const float *d_emit, int n, int T,
                    const float *d_grad_pos, const float *d_D, void *d_scratch,
                    size_t scratch_bytes, double *d_dD, void *stream);

/* ---------------------------------------------------------------------------
 * Differentiable Born-Wolf image (new: the reference has no gradients).  The
 * reference's Born-Wolf image (overlay_signal_ with the 1-nm depth-keyed
 * grids, src/scopyon/_epifm.py:76-126, :181-213, :224-282) made continuous:
 * each grid value fills a 1-nm cell and a pixel integrates that
 * piecewise-constant function exactly (bilinear interpolation of the grid's
 * 2-D prefix sum at the pixel corners, evaluated in FP64 from the quadrant
 * tables of sc_psf_quadrant_sat); the two depth keys around
 * |z - z_focal| / res are blended linearly (the last key, key_hi, beyond the
 * cutoff); TIRF excitation A(z) = exp(-|z - z_focal| inv_pen) (:1281-1289):
 *   mu[f][i][j] = bg[f] + sum_e I_e A(z_e) cnorm B_e(i, j).
 * Emitters are float4 (x, y: metres from the image centre; z; I: photons),
 * [n_frames][n_emit].                                                        */
typedef struct {
    int32_t nw, nh, n_frames, n_emit;
    int32_t n_r, sat_pitch;  /* quadrant tables: (n_r + 1) rows of sat_pitch float2  */
    int32_t key_hi;          /* depth keys 0 .. key_hi have tables (key_hi = cutoff / res) */
    int32_t pad;
    double px, res, inv_pen, z_focal;
    double cnorm;            /* psf_normalization * res^2                              */
    const int32_t *d_key_slot; /* table slot of each depth key (-1: not built)         */
} ScBWParams;

/* FP64 work buffer of sc_bw_forward: n_frames * nw * nh doubles. */
size_t sc_bw_work_bytes(const ScBWParams *p);

/* Forward: d_mu [n_frames][nw][nh] FP32 (FP64 accumulation in d_work). */
int sc_bw_forward(const ScBWParams *p, const float *d_emit, const float *d_bg, const float *d_sat,
                  void *d_work, size_t work_bytes, float *d_mu, int32_t *d_status, void *stream);

/* Adjoint: d_grad_emit [n_frames][n_emit] float4 = (dL/dx, dL/dy, dL/dz, dL/dI)
 * from d_grad_mu = dL/dmu; each emitter's sums in a fixed order.  dL/dbg is
 * the per-frame sum of dL/dmu (sc_segment_sum).                              */
int sc_bw_backward(const ScBWParams *p, const float *d_emit, const float *d_sat,
                   const float *d_grad_mu, float *d_grad_emit, int32_t *d_status, void *stream);

/* Largest tile count (tiles per image x images) sc_bin_steps_static takes. */
#define SC_BIN_STATIC_MAX_TILES 65536

/* sc_bin_steps without a caller workspace: the per-bin counts and cursors
 * live in a fixed 1 MiB device array inside the library (room for
 * SC_BIN_STATIC_MAX_TILES tiles; more returns SC_ERR_ARG).  For callers that
 * cannot allocate device memory -- a C or FFI host handed only the record and
 * output buffers, or a frame loop that must not allocate -- it calls no
 * allocator.  The first call on a device looks up the array's address with
 * that device current; make that first call before any stream capture.  The
 * address is kept for the life of the process, so the device's primary
 * context must not be reset (cudaDeviceReset) while the library is loaded.
 * Records with a negative first pixel are not binned and set status bit 6.  The
 * array is shared by every call on a device: calls that overlap in time (on
 * different streams or host threads) race on it and must be serialised.
 * No counterpart in the reference, which bins nothing
 * (src/scopyon/_epifm.py:1262-1264).                                        */
int sc_bin_steps_static(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                        int32_t *d_tile_start, int32_t *d_items, int32_t *d_status,
                        void *stream);

/* FP64 splat for the injected-draws parity mode: every record's footprint,
 * each pixel's slice sum from the double-float quadrant tables evaluated in
 * FP64, times res^2 and the record's FP64 normalisation d_norm[r] (from
 * sc_emitter_steps), added to d_image (n_images x nw x nh FP64, zeroed by
 * the caller) with FP64 atomic adds when the slice sum is positive.  A warp
 * per record, no binning; records need not be sorted.  The expected image
 * then matches an FP64 evaluation of overlay_signal_
 * (src/scopyon/_epifm.py:224-282) to ~1e-13 relative, so that draws the
 * camera takes from the expectation (the EMCCD inverse CDF) are the
 * reference's.                                                              */
int sc_splat_fp64(const ScStepRec *d_recs, const double *d_norm, int n_rec, const float *d_sat,
                  const ScSplatParams *p, double *d_image, int32_t *d_status, void *stream);

/* Work plan of the persistent batched frame (sc_batch_frame): fields of view
 * packed into one canvas, and the order in which the launch's blocks take
 * work.  A work entry w >= 0 is tile w (its box and summed-area records
 * into its tile buffer); w < 0 is chunk -w - 1 (chunk_pixels pixels of one
 * field: the merge of the covering tile buffers).  Every tile a field's
 * pixels read must come before that field's chunks in the list.             */
typedef struct {
    const int32_t *d_work;          /* [n_work] tile indices and -(chunk + 1)         */
    const int32_t *d_tile_field_off;/* [n_tiles + 1] CSR: fields whose pixels read   */
    const int32_t *d_tile_field;    /*   tile t's buffer (their counters it advances) */
    const int32_t *d_field;         /* [n_fields][4]: first pixel i0, j0, edge, and   */
                                    /*   the number of tiles its pixels read          */
    const int32_t *d_chunk;         /* [n_chunks][2]: field, first pixel in the field */
    int32_t *d_counters;            /* [2 + n_fields]: next work entry, stop flag,    */
                                    /*   tiles done per field; zeroed by the call     */
    int32_t n_work, n_fields, n_chunks, chunk_pixels;
    int32_t spin_limit;             /* polls of a chunk's wait for its tiles (0: about */
                                    /*   a second's worth)                            */
    int32_t target_extra;           /* test hook: added to every field's tile count,  */
                                    /*   so that the waits run out (status bit 5)     */
    int32_t blocks_per_sm;          /* resident blocks per SM (0: as many as fit);    */
                                    /*   fewer leave room for work on other streams   */
    int32_t pad;
} ScBatchPlan;

/* Persistent batched frame: one launch of resident blocks that take work
 * entries in plan order from a device counter.  A tile entry splats the
 * tile's box records (bulk copies, as sc_splat) and summed-area records into
 * its tile buffer in d_ws (sc_splat_workspace_bytes) and advances the tile
 * counters of the fields that read it; a chunk entry waits (bounded poll)
 * until its field's tiles are done, then merges its pixels into d_expect.
 * A second launch then draws the native camera (d_poisson_table required)
 * on the fields' pixels, the expectation replacing the photons.  The
 * wait always ends: a field's tiles are taken before its chunks, and a
 * block that took a tile finishes it without waiting on anything.  Per
 * pixel, the results equal sc_splat followed by sc_camera on the canvas
 * (same sums in the same order, same draws); pixels outside the fields are
 * not written.  Replaces the per-field loop of generate_frames
 * (src/scopyon/_epifm.py:1045-1049) for many fields.  Box tables with 12..16
 * pixel offsets per axis only (else SC_ERR_ARG).                            */
int sc_batch_frame(const ScStepRec *d_recs, const int32_t *d_tile_start, const int32_t *d_items,
                   const float *d_sat, const float *d_box, const ScSplatParams *sp,
                   const ScBatchPlan *plan, const ScCameraParams *cp, const float *d_offset_f,
                   const float *d_inv_gain_f, const float *d_sigma, const double *d_table_value,
                   const double *d_table_cdf, void *d_ws, size_t ws_bytes, float *d_expect,
                   float *d_adc32, int32_t *d_status, void *stream);

/* Bytes of scratch sc_splat needs: one FP32 (tile + halo)^2 buffer per tile. */
size_t sc_splat_workspace_bytes(const ScSplatParams *p);

/* Splat: each CTA sums the whole footprints of the records binned to its
 * tile into a (tile + halo)^2 buffer in shared memory and stores it in the
 * workspace; a second pass adds the overlapping buffers into d_image
 * (d_image NULL: no second pass, the caller merges the workspace with
 * sc_merge_camera).  Replaces overlay_signal_ (src/scopyon/_epifm.py:224-282)
 * for every particle and sub-step.                                          */
int sc_splat(const ScStepRec *d_recs, const int32_t *d_tile_start,
             const int32_t *d_items, const float *d_sat, const float *d_box,
             const ScSplatParams *p, void *d_ws, size_t ws_bytes, float *d_image,
             int32_t *d_status, void *stream);

/* The merge of sc_splat and the native camera of sc_camera in one pass, for
 * one image: for each pixel the photons are the sum of the workspace's tile
 * buffers that cover it (d_ws of a sc_splat call with d_image NULL, same
 * splat params), in the order sc_splat's merge adds them; then the camera
 * as sc_camera draws it (cp->exact 0).  d_expect (may be NULL) and d_adc32
 * equal those of sc_splat with an image followed by sc_camera, bit for bit,
 * without the photon image's write and read.  Replaces the same reference
 * lines as the two (src/scopyon/_epifm.py:224-282, :1430-1484).           */
int sc_merge_camera(const ScSplatParams *sp, const void *d_ws, size_t ws_bytes,
                    const ScCameraParams *cp, const float *d_offset_f,
                    const float *d_inv_gain_f, const float *d_sigma,
                    const double *d_table_value, const double *d_table_cdf, float *d_expect,
                    float *d_adc32, int32_t *d_status, void *stream);

/* Camera model and ADC.  Replaces _EPIFMSimulator.__detector_output, the
 * EMCCD / CCD / CMOS classes and __get_analog_to_digital_converter_counts
 * (src/scopyon/_epifm.py:329-433, :1430-1484).
 * Native mode (p->exact == 0): Philox draws, FP32 arithmetic with the float
 * maps d_offset_f / d_inv_gain_f (NULL: constants offset0 / 1/gain0).  Each
 * pixel pair shares one Philox4x32-10 block (counter: the pair index and the
 * frame counter): one 32-bit word per pixel for its Poisson draw, which takes
 * no rejection below a mean of 256 (table inversion of the integer part, then
 * sequential inversion of the fraction at the word's residual in its bin),
 * and a Box-Muller pair for the two read-noise normals; a pixel's draws so
 * depend on its index and the frame only.  The EMCCD output follows the
 * reference's truncated discrete law.
 * Exact mode (p->exact == 1): draws injected by the caller — d_inj_signal
 * (electrons) and d_inj_noise (electrons) or, for the CMOS table,
 * d_inj_uniform — and the reference's FP64 ADC sequence with d_offset /
 * d_gain.  Writes the expectation QE*(photons+background) to d_expect and
 * the ADC image to d_adc64 and/or d_adc32.                                  */
int sc_camera(const ScCameraParams *p, const float *d_photons,
              const double *d_offset, const double *d_gain,
              const float *d_offset_f, const float *d_inv_gain_f, const float *d_sigma,
              const double *d_table_value, const double *d_table_cdf,
              const double *d_inj_noise, const double *d_inj_signal,
              const double *d_inj_uniform, float *d_expect, double *d_adc64,
              float *d_adc32, int32_t *d_status, void *stream);

/* Poisson tables for the camera's native draws: for every integer mean j <
 * 256, the Poisson(j) CDF as 32-bit fixed point (summed in FP64) and a guide
 * of starting points for its inversion.  Built once per device into a caller buffer of
 * sc_poisson_table_bytes() bytes (16-byte aligned), read by sc_camera
 * (ScCameraParams.d_poisson_table).  Replaces the Poisson draws of
 * CCD / CMOS get_signal and the photo-electron count inside the EMCCD law
 * (src/scopyon/_epifm.py:348-353, :365-400, :428-433).                      */
size_t sc_poisson_table_bytes(void);
int sc_poisson_table(void *d_table, size_t bytes, void *stream);

/* Exact EMCCD draw: the reference's discrete distribution over integer
 * output electrons, inverse CDF at the given uniform, per pixel
 * (EMCCD.probability_distribution / draw_signal, src/scopyon/_epifm.py:365-400). */
int sc_emccd_exact(const double *d_photons, double qe, double background,
                   const double *d_uniform, int n_pixels, double emgain,
                   double *d_signal, int32_t *d_status, void *stream);

/* Laplacian-of-Gaussian scale space for blob detection (the blob_log search
 * of spot_detection, src/scopyon/analysis/spot_detection.py:14-46).  For
 * scale s: d_cube[(i * nh + j) * n_scales + s] = -sigma_s^2 times the sum
 * over both axes of (second-derivative kernel along that axis, Gaussian
 * kernel along the other) applied to d_img (nw x nh FP64), with the kernels
 * d_phi / d_d2 of scale s at d_tap_off[s] .. + 2 d_radius[s] and scipy.ndimage's
 * 'reflect' edges; FP64.  d_work: 2 * nw * nh * n_scales doubles.           */
int sc_log_cube(const double *d_img, int nw, int nh, const double *d_phi, const double *d_d2,
                const int32_t *d_tap_off, const int32_t *d_radius, const double *d_sigma,
                int n_scales, double *d_work, size_t work_bytes, double *d_cube, void *stream);

/* Blobs of the scale space: cells above threshold that are the maximum of
 * their 3 x 3 x 3 neighbourhood, written as (i, j, s) int32 triples to
 * d_peaks (at most capacity; *d_count receives how many were found, in no
 * particular order).                                                        */
int sc_log_peaks(const double *d_cube, int nw, int nh, int n_scales, double threshold,
                 int32_t *d_count, int32_t *d_peaks, int capacity, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SCOPYON_GB300_H */
