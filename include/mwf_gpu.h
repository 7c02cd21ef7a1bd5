/*
 * mwf_gpu.h -- C ABI of the GB300 (sm_103a) Model Waleffe Flow timestep.
 *
 * Plain C types only (ints, doubles, pointers, sizes).  Every entry point returns 0 on
 * success or a negative MWF_ERR_* code; mwf_last_error() gives the message of the last
 * failure on the calling thread.  A handle owns the device state of one or more
 * independent runs and is not re-entrant: use one handle per host thread.
 *
 * Layout of host state arrays: exactly the reference's `type(mpt)` arrays
 * (program/variables.f90:12-15): two arrays `re` and `im` of K*M*NN doubles each, Fortran
 * order (K, 0:M-1, 0:NN-1), K = 2*K0-1 wall-normal components, M = 2*MM-1 x slots (slot
 * m > MM-1 holds wavenumber m-M), NN z wavenumbers.  A Fortran caller passes
 * c_loc(vel_c%Re) and c_loc(vel_c%Im).
 */
#ifndef MWF_GPU_H
#define MWF_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { MWF_FP64 = 0, MWF_FP32 = 1 };

enum {
  MWF_OK = 0,
  MWF_ERR_ARG = -1,      /* invalid argument (null pointer, run index, flag)            */
  MWF_ERR_SIZE = -2,     /* grid size not supported (MM, NN must be 2^a 3^b, limits)   */
  MWF_ERR_CUDA = -3,     /* a CUDA runtime call failed                                  */
  MWF_ERR_NOMEM = -4,    /* device memory allocation failed                             */
  MWF_ERR_DEVICE = -5,   /* a kernel recorded an internal inconsistency                 */
  MWF_ERR_NONFINITE = -6 /* the state of a run contains NaN/Inf                         */
};

/* One run: the runtime copy of the reference's compile-time parameters
 * (program/parameters.f90:7-72).  theta is in radians (d_theta). */
typedef struct mwf_run_desc {
  int K0;          /* wall-normal modes: 4 (M4) or 6 (M6)                      i_K0     */
  int MM;          /* x modes: |m| < MM, physical x grid 3*MM                  i_MM     */
  int NN;          /* z modes: 0 <= n < NN, physical z grid 3*NN               i_NN     */
  int precision;   /* MWF_FP64 (plain path) or MWF_FP32                                 */
  double alpha;    /* 2 pi / Lx                                                d_alpha  */
  double gamma;    /* 2 pi / Lz                                                d_gamma  */
  double Re;       /* Reynolds number                                          d_Re     */
  double dt;       /* time step                                                d_dt     */
  double drag;     /*                                                          d_drag   */
  double vdrag;    /*                                                          d_vdrag  */
  double hypo;     /* hypo-viscosity coefficient                               d_HYPO   */
  int dragall;     /* 1: drag on every wall-normal mode                        s_dragall*/
  int reflect;     /* symmetry masks applied before each step (velocity.f90:68-74)     */
  int uvreflect;
  int wreflect;
  double theta;    /* base-flow angle in radians                               d_theta  */
  /* Tuning knobs, 0 = the planner's default (chosen by mwf_gb300.autotune by timing):
   * columns per x-forward / x-inverse work item, x lines per z-pass work item, and the
   * largest FFT radix of the x and z transforms (8, 12 or 16; capped per pass and
   * precision).  No counterpart in the reference, whose FFTW plans are tuned at start-up
   * by FFTW itself (transform.fftw5.f90:33-59, flag FFTW_PATIENT). */
  int xf_cols;
  int xi_cols;
  int z_lines;
  int x_radix;
  int z_radix;
} mwf_run_desc;

typedef struct mwf_handle mwf_handle;

/* Allocate device state for n_runs runs on `device` and build their plans and FP64
 * implicit-update tables.  Replaces vel_precompute + var_precompute + var_LHSRHS +
 * tra_precompute (velocity.f90:43-50, variables.f90:488-533,565-597,
 * transform.fftw5.f90:33-59).  The state of every run starts at zero with the Euler
 * start flag set (nst = .true.). */
int mwf_create(const mwf_run_desc* runs, int n_runs, int device, mwf_handle** out);
int mwf_destroy(mwf_handle* h);

/* Copy a run's MPT state in (vel_c <- host) / out (host <- vel_c).  Replaces the
 * io_load_mpt / io_save_mpt data movement (io.f90:166-204, 306-340). */
int mwf_set_state(mwf_handle* h, int run, const double* re, const double* im);
int mwf_get_state(mwf_handle* h, int run, double* re, double* im);

/* Advance every run by nsteps steps: vel_imposesym + vel_TS (main.f90:22-24,
 * velocity.f90:21-41) per step, replayed as a CUDA graph.  Synchronous at return. */
int mwf_step(mwf_handle* h, int nsteps);

/* Same as mwf_step but returns once the work is queued on the handle's stream. */
int mwf_step_async(mwf_handle* h, int nsteps);
int mwf_synchronize(mwf_handle* h);

/* The AB2 history of a run (the previous nonlinear term, vel_onl of velocity.f90:16) in the
 * state's layout, and its Euler-start flag (1: the next step is an Euler step).  With
 * mwf_get_state / mwf_set_state they checkpoint a run exactly: restored into any handle (of the
 * same model, grid and precision) it continues bitwise as it would have.  The reference keeps
 * the history only in memory (its state files hold vel_c alone). */
int mwf_get_history(mwf_handle* h, int run, double* re, double* im, int* euler_next);
int mwf_set_history(mwf_handle* h, int run, const double* re, const double* im, int euler_next);

/* *idle = 1 when every step queued on the handle (mwf_step_async) has finished, 0 otherwise;
 * does not wait and does not check the kernels' error flags (mwf_synchronize does). */
int mwf_query(mwf_handle* h, int* idle);

/* Set the Euler-start flag of a run (the reference's nst = .true. after a restart:
 * the AB2 history is not part of the state file, velocity.f90:24-27,48). */
int mwf_reset_history(mwf_handle* h, int run);

/* Physical-space diagnostics of a run's current state, on the device: the u,v,w fields
 * without the base flow are transformed to the 3MM x 3NN grid (vel_mpt2phys,
 * velocity.f90:84-90), epos (the y-mean of u^2+v^2+w^2, velocity.f90:115-126) is formed at
 * every point, and the call returns the number of points with epos > threshold (the count
 * of io_writeVTK_txz, io.f90:597-615, on the full grid) and the physical-space energy
 * sum(epos)/(3MM*3NN) of vel_energy (velocity.f90:144-162).  The reference divides the count
 * by (3MM+1)(3NN+1) to get its turbulent fraction (io.f90:615). */
int mwf_phys_diagnostics(mwf_handle* h, int run, double threshold, double* count_above, double* energy);

/* Stop (active = 0) or resume (1) stepping one run of a handle; the other runs are not
 * affected.  Used by a server to retire a finished request inside a running batch.  There is
 * no counterpart in the reference, which runs one simulation per process. */
int mwf_set_active(mwf_handle* h, int run, int active);

/* Test only: make the bounded wait of the staged FP32 z pass (the variant selected by a z radix
 * cap, whose input rows are staged in shared memory by bulk copies completing on an mbarrier)
 * run out on purpose.  Each staging barrier of run `run` is armed with extra_bytes (a multiple
 * of 16) more than its copies carry, and a barrier phase is waited for at most wait_ms
 * milliseconds (0: the default of about a second).  A step then returns MWF_ERR_DEVICE with the
 * copy-timeout flag (0x8) in its message, every CTA having completed the extra bytes itself and
 * waited for its real copies before leaving; the handle's state is undefined after that, other
 * handles are not affected.  extra_bytes = 0 and wait_ms = 0 restore normal operation.  No
 * counterpart in the reference (failure detection of the device code). */
int mwf_test_copy_timeout(mwf_handle* h, int run, unsigned extra_bytes, double wait_ms);

/* Perturbation kinetic energy of vel_energy(vel_mpt2phys(vel_c)) (velocity.f90:84-90,
 * 144-162), computed in FP64 with compensated sums. */
int mwf_energy(mwf_handle* h, int run, double* e);

/* Physical velocity field of a run, vel_mpt2phys (velocity.f90:84-90: var_mpt2spec then
 * tra_spec2phys, transform.fftw5.f90:64-87), without the base flow, as the reference's
 * type(phys) array Re(KK, 0:3NN-1, 0:3MM-1): p has KK*3NN*3MM doubles with the field index
 * fastest, then z, then x.  Serves turb.f90:45 and the VTK writers of io.f90. */
int mwf_get_phys(mwf_handle* h, int run, double* p);

/* Spectrum maxima of io_save_Uspec (io.f90:345-372): for the u,v,w spectral coefficients
 * of the current state (var_mpt2spec, no base flow), m_max[|m|] (MM values) and n_max[n]
 * (NN values) are the largest moduli sqrt(re^2 + im^2) over k and the other wavenumber:
 * the two columns of vel_spec%04d.dat. */
int mwf_spectrum_maxima(mwf_handle* h, int run, double* m_max, double* n_max);

/* Velocity probes of vel_history (velocity.f90:164-180) as written by io_write_history
 * (io.f90:473-483): for j = 0..n_probes-1 the point x = 0, z index ji = j*3NN/n_probes + 1
 * (integer division), height y; H[4j..4j+3] = (ji*Lz/(3NN), u, v, w) with velU, velV, velW
 * of modes.M4.f90:83-107 / modes.M6.f90:81-111 and Lz = 2 pi / gamma.  The reference uses
 * n_probes = i_H = 32 (parameters.f90:41) and y = 0.  1 <= n_probes < 3NN. */
int mwf_history(mwf_handle* h, int run, double y, int n_probes, double* H);

/* x-resolution remap of var_quadX (variables.f90:168-185) for any factor >= 1: the
 * coefficient of x wavenumber m moves to factor*m; what lands outside |m| <= MM-1 is
 * dropped and the rest is zero.  factor = 2 is var_doubleX (variables.f90:147-165) with the
 * mirror index of var_quadX for negative m: the reference's var_doubleX indexes
 * M - 2(m - M), past the end of its array.  As in the reference, with factor > 1 dividing MM
 * the wavenumber -MM lands in slot MM-1 and replaces the positive mode there.  Sets the
 * Euler-start flag (the remapped state has no AB2 history). */
int mwf_remap_x(mwf_handle* h, int run, int factor);

/* State blend of utils/interpstate.f90:32-33: c[run] := (1-d) c[run] + d c[other], each
 * product and the sum rounded separately.  The runs must have the same model, MM, NN and
 * precision.  Sets the Euler-start flag of run. */
int mwf_blend_state(mwf_handle* h, int run, int other, double d);

/* Additive noise of var_randadd (variables.f90:253-269): scale*r is added to the real and
 * the imaginary part of every coefficient with m != 0 and n != 0, r uniform in [0, 1).
 * The reference draws r with Fortran's RANDOM_NUMBER; this call draws it from SplitMix64 of
 * (seed, coefficient index), so a given seed gives the same state on every device.  The AB2
 * history is kept (call mwf_reset_history for the reference's restart semantics). */
int mwf_add_noise(mwf_handle* h, int run, double scale, unsigned long long seed);

/* Advance nsteps steps and return the device time of the whole sequence in milliseconds,
 * measured with CUDA events recorded on the handle's stream around the graph launches. */
int mwf_step_timed(mwf_handle* h, int nsteps, double* ms);

/* Launch the step's passes one by one, nreps times, with CUDA events around each launch
 * on the handle's stream; ms_per_pass[0..2] receive the mean device time per step of the
 * x-forward, z (transforms + nonlinear) and x-inverse (+ update) passes.  Advances the
 * state by nreps steps. */
int mwf_profile_passes(mwf_handle* h, int nreps, double* ms_per_pass);

/* Step mode of a handle.  on = 1: the FP32 runs whose three passes all have batched forms step
 * in one persistent launch per step -- resident CTAs take the x-forward, z and x-inverse items of
 * all those runs from one ticket counter, an item waiting (bounded) until its run's previous pass
 * is done; on = 0 (the default): one launch per pass and grid size.  Both modes give bitwise the
 * same results.  On GB300 the per-pass launches are faster (the z pass needs 111 KB of shared
 * memory per CTA, which holds every item of the persistent launch to two CTAs per SM).  No
 * counterpart in the reference. */
int mwf_set_persistent(mwf_handle* h, int on);

/* Number of kernel launches one step of the handle makes (the passes, grouped over runs,
 * plus one launch per symmetry mask of each run that has one). */
int mwf_kernels_per_step(mwf_handle* h, int* n);

/* Measured arithmetic peak of the current device: which = 0 FP64 FMA, 1 FP32 FMA.
 * Returns TFLOP/s (2 flops per FMA). */
int mwf_measure_fma_peak(int device, int which, double* tflops);

/* Time step for callers that cannot allocate device memory.  This entry point has no
 * counterpart in the reference.  It is meant for host codes that own every device buffer
 * themselves (CUDA Fortran or OpenACC device arrays, a caller-managed pool) or may not
 * grow their device footprint after start-up, so they cannot let the library cudaMalloc
 * its own state as mwf_create does.
 *
 * c_re, c_im (the MPT state) and onl_re, onl_im (the AB2 history) are DEVICE pointers of
 * the current device, each K*M*NN doubles in the reference layout described above; they
 * are read and updated in place.  first_step = 1 starts with the Euler step (the
 * reference's nst = .true.) and ignores the history on input.  The call advances nsteps
 * steps on the legacy default stream of the current device and returns when they are done.
 *
 * All intermediates live in one fixed file-scope device array of 64 MiB; every GPU that
 * loads the library's module holds it until the process exits.  Runs whose intermediates
 * exceed it (about 16 * (5*KK*3MM*NN + 3*K*M*NN) bytes in FP64) fail with MWF_ERR_SIZE;
 * for example M4 fits up to MM = NN = 128 in FP64.  Both precisions are supported: the
 * FP32 form keeps its implicit-update tables in the form the FP32 passes read (as
 * mwf_create builds them).  Every call looks up the array's device address on the current
 * device with cudaGetSymbolAddress.  The call makes no cudaMalloc, cudaFree or other
 * allocating call.  Every call shares the array and rewrites the parts it reads (tables,
 * twiddles, descriptor, error word): calls that overlap on the GPU (other host threads, or
 * other streams) race and must be serialised by the caller.  If a pass records an internal
 * error the call returns MWF_ERR_DEVICE and leaves the caller's arrays unchanged.
 * Symmetry masks are not supported here (MWF_ERR_ARG). */
int mwf_step_noalloc(const mwf_run_desc* d, double* c_re, double* c_im, double* onl_re,
                     double* onl_im, int first_step, int nsteps);

/* The stand-alone 2D transforms of the reference's transform module on fields the caller
 * supplies, FP64 on the current device (the run descriptor gives K0, MM, NN; its other fields
 * are ignored).  mwf_spec2phys is tra_spec2phys (transform.fftw5.f90:64-87): the KK spectral
 * fields s_re/s_im, type(spec) layout (KK, 0:M-1, 0:NN-1), padded by the 3/2 rule and
 * transformed backward (unnormalised, FFTW's e^{+i} and c2r conventions) to p, type(phys)
 * layout (KK, 0:3NN-1, 0:3MM-1).  mwf_phys2spec is tra_phys2spec (transform.fftw5.f90:
 * 122-145): p scaled by 1/(3MM 3NN), transformed forward and truncated to |m| <= MM-1,
 * n < NN.  Each call allocates its device buffers and frees them before returning.
 * 3NN <= 3072. */
int mwf_spec2phys(const mwf_run_desc* d, const double* s_re, const double* s_im, double* p);
int mwf_phys2spec(const mwf_run_desc* d, const double* p, double* s_re, double* s_im);

/* Number of complex MPT coefficients of a run: K*(2MM-1)*NN (the "dof" of dof-steps/s). */
long long mwf_run_dof(const mwf_run_desc* d);

/* Device bytes a handle with these runs would allocate (admission control). */
long long mwf_footprint_bytes(const mwf_run_desc* runs, int n_runs);

/* How the library would step one run: the kernels of its three passes and their tiling, as the
 * planner of mwf_create chooses them (host only: no device is needed).  batched_* = 1 selects
 * the FP32 kernels with compile-time plans (subset-split x passes, batched z pass), 0 the
 * kernels with run-time plans.  *_ctas_per_sm is the occupancy a batched kernel is compiled for
 * (0 for the others).  Returns MWF_OK, or MWF_ERR_SIZE / MWF_ERR_ARG (with mwf_last_error) for a
 * run the kernels cannot take.  Not part of the reference's interface: an observability aid. */
typedef struct mwf_run_plan {
  int batched_x, batched_z;
  int xf_cols, xi_cols;          /* columns of an x-forward / x-inverse work item */
  int z_lines;                   /* x lines of a z work item */
  int xf_ctas_per_sm, z_ctas_per_sm, xi_ctas_per_sm;
  long long xf_smem, z_smem, xi_smem;   /* dynamic shared memory of a CTA, bytes */
  int xf_items, z_items, xi_items;      /* work items of one step */
} mwf_run_plan;
int mwf_describe_run(const mwf_run_desc* d, mwf_run_plan* out);

/* Pinned host memory for fast state copies. */
int mwf_host_alloc(size_t bytes, void** p);
int mwf_host_free(void* p);

/* Message of the last error on this thread (empty if none).  Returns the message length. */
int mwf_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* MWF_GPU_H */
