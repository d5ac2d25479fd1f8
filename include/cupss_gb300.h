/* C-ABI of the GB300-native cuPSS pseudospectral step.
 *
 * Two levels, both plain C (no C++ or torch types in the signatures):
 *
 *  1. Solver level (cupssgb_solver_*): a system given directly as the parser's
 *     intermediate representation -- fields, implicit q-monomials, explicit terms
 *     (product of fields x sum of q-monomials) and noise amplitudes.  This is the
 *     seam the reference's host classes drive through their extern "C" launchers
 *     (inc/cupss/field_kernels.cuh:7-19, inc/cupss/term_kernels.cuh:7-15) plus
 *     cuFFT/cuRAND (src/field.cpp:247-316, src/term.cpp:48-64); here one call
 *     advances whole time steps.
 *
 *  2. Evolver level (cupssgb_evolver_*): the reference's public C++ API
 *     (inc/cupss/evolver.h:14-86) -- string equations parsed by the library --
 *     flattened to C for FFI callers (ctypes, cgo, JNI).
 *
 * Conventions: every function returns 0 on success or a negative status
 * (CUPSSGB_ERR_*); cupssgb_last_error() gives the message of the last failure on
 * the calling thread.  Real fields are sx*sy*sz floats indexed k*sx*sy + j*sx + i
 * (the reference's index, src/field.cpp:102).  Fourier fields are the reference's
 * full complex layout: 2*sx*sy*sz floats (re, im) at the same index, unnormalised
 * forward transform of the real field (cuFFT/FFTW convention).
 * Grid sizes: powers of two, 2 <= sx <= 2048, 1 <= sy, sz <= 1024.
 * One CUDA stream per handle; handles are independent and hold no global state.
 */
#ifndef CUPSS_GB300_H
#define CUPSS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define CUPSSGB_OK 0
#define CUPSSGB_ERR_INVALID (-1)
#define CUPSSGB_ERR_CUDA (-2)
#define CUPSSGB_ERR_UNSUPPORTED (-3)
#define CUPSSGB_ERR_STATE (-4)
#define CUPSSGB_ERR_PARSE (-5)
#define CUPSSGB_ERR_LIMIT (-6)

/* Same members and layout as the reference's struct pres (inc/cupss/defines.h:31-39). */
typedef struct cupssgb_pres {
  float preFactor;
  int q2n;
  int iqx;
  int iqy;
  int iqz;
  int invq;
} cupssgb_pres;

typedef struct cupssgb_solver cupssgb_solver;
typedef struct cupssgb_evolver cupssgb_evolver;

/* Message of the last failed call on this thread ("" if none). */
const char* cupssgb_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int cupssgb_version(void);

/* ---------------- solver level ---------------- */

/* Replaces the per-field/per-term allocation and plan creation of
 * field::common_constructor / term::common_constructor (src/field_init.cpp:15-154,
 * src/term_init.cpp:11-71).  dx, dy, dz: cell sizes; dt: time step. */
int cupssgb_solver_create(int sx, int sy, int sz, float dx, float dy, float dz, float dt,
                          cupssgb_solver** out);
int cupssgb_solver_destroy(cupssgb_solver* s);

/* evolver::createField (src/evolver.cpp:177-196).  Returns the field index (>= 0). */
int cupssgb_solver_add_field(cupssgb_solver* s, int dynamic);
/* field::implicit as built by parser::add_equation (src/parser.cpp:681-738):
 * dynamic fields get the LHS prefactors negated, non-dynamic ones as written. */
int cupssgb_solver_set_implicit(cupssgb_solver* s, int field, const cupssgb_pres* pres, int n);
/* evolver::createTerm (src/evolver.cpp:326-362): product = field indices
 * (multiset, n_product >= 0), pres = the term's prefactor list.  Returns the term
 * index within the field (>= 0). */
int cupssgb_solver_add_term(cupssgb_solver* s, int field, const int* product, int n_product,
                            const cupssgb_pres* pres, int n_pres);
/* field::updateParameter / term::precomputePrefactors (src/field.cpp:422-441,
 * src/term_init.cpp:135-200): new prefactors for an existing term (same count). */
int cupssgb_solver_set_term_pres(cupssgb_solver* s, int field, int term, const cupssgb_pres* pres,
                                 int n);
/* Implicit prefactors may be replaced after prepare (field::precalculateImplicit). */
int cupssgb_solver_update_implicit(cupssgb_solver* s, int field, const cupssgb_pres* pres, int n);
/* evolver::addNoise (src/evolver.cpp:162-171); amp = NULL switches noise off. */
int cupssgb_solver_set_noise(cupssgb_solver* s, int field, const cupssgb_pres* amp);
/* Seed of the counter-based noise (the reference seeds cuRAND with time(NULL),
 * src/field_init.cpp:137). */
int cupssgb_solver_set_seed(cupssgb_solver* s, unsigned long long seed);

/* Replaces field::prepareDevice + precalculateImplicit + term::prepareDevice
 * (src/field_init.cpp:215-284, src/term_init.cpp:108-200): compiles the step
 * plan and allocates device state.  All fields start at zero. */
int cupssgb_solver_prepare(cupssgb_solver* s);
/* Initial condition: copyHostToDevice + toComp of evolver::prepareProblem
 * (src/evolver.cpp:114-117).  host_real: sx*sy*sz floats.  From page-locked memory
 * (cupssgb_host_alloc) the copy is asynchronous, on an input stream of its own that
 * overlaps work queued earlier (host_real must stay unchanged until the solver's next
 * synchronising call); from pageable memory it completes before the call returns. */
int cupssgb_solver_set_real(cupssgb_solver* s, int field, const float* host_real);
/* Same from a device pointer (stream-ordered on the solver's stream). */
int cupssgb_solver_set_real_device(cupssgb_solver* s, int field, const float* dev_real);
/* nsteps x evolver::advanceTime (src/evolver.cpp:199-226), asynchronous. */
int cupssgb_solver_advance(cupssgb_solver* s, int nsteps);
/* Real-space field (field::real_array after the last step, src/field.cpp:64-66). */
int cupssgb_solver_get_real(cupssgb_solver* s, int field, float* host_real);
int cupssgb_solver_get_real_device(cupssgb_solver* s, int field, float* dev_real);
/* Fourier-space field (field::comp_array, full complex layout, 2*N floats). */
int cupssgb_solver_get_fourier(cupssgb_solver* s, int field, float* host_complex);
int cupssgb_solver_get_fourier_device(cupssgb_solver* s, int field, float* dev_complex);
/* Materialisation points for user callbacks (field::callback / callbackFourier,
 * src/field.cpp:48-86).  advance_phase runs one half of a time step: phase 0 updates
 * the non-dynamic fields, phase 1 the dynamic ones and counts the step (advance(1) ==
 * phase 0 + phase 1).  Between phases a caller can read a field in the reference's
 * device layouts, modify it and write it back:
 *   get_real_pairs_device      real field as N float2 (x, 0)          (real_array_d)
 *   get_dealiased_pairs_device dealiased real field as N float2 (x, 0) (real_dealiased_d)
 *   set_fourier_device         full complex spectrum, 2N floats       (comp_array_d);
 *                              projected onto real fields, dealiased copy re-derived
 *   set_real_pairs_device      real field (+ optional dealiased copy, NULL = re-derive)
 * All are ordered on the solver's stream. */
int cupssgb_solver_advance_phase(cupssgb_solver* s, int phase);
int cupssgb_solver_get_real_pairs_device(cupssgb_solver* s, int field, float* dev_pairs);
int cupssgb_solver_get_dealiased_pairs_device(cupssgb_solver* s, int field, float* dev_pairs);
int cupssgb_solver_set_fourier_device(cupssgb_solver* s, int field, const float* dev_complex);
int cupssgb_solver_set_real_pairs_device(cupssgb_solver* s, int field, const float* dev_pairs,
                                         const float* dev_dealiased_pairs);
/* Waits for all work queued on the solver: its stream, and the input copies and output
 * copies (cupssgb_solver_snapshot_real) on their own streams. */
int cupssgb_solver_synchronize(cupssgb_solver* s);
/* Output path of writeOut (src/field.cpp:350-402): copies the real values of a field into
 * host memory without stalling the step.  The field is materialised on the solver's
 * stream into a staging buffer of its own (allocated on first use);
 * the device-to-host copy runs on a separate output stream, so steps queued after this
 * call overlap with it.  done_event (a cudaEvent_t, may be NULL) is recorded on the
 * output stream once host_real holds the values; host_real should be page-locked
 * (cupssgb_host_alloc) for the copy to be asynchronous.  Each field has two staging
 * buffers, used in turn, so that a snapshot's transform overlaps the previous snapshot's
 * copy; a snapshot waits until the copy two snapshots back has left its buffer. */
int cupssgb_solver_snapshot_real(cupssgb_solver* s, int field, float* host_real, void* done_event);
/* Scheduling priority of the solver's work: 0 (the default) or higher levels, whose
 * kernels' CTAs the GPU schedules first when several streams compete (clamped to the
 * device's priority range).  Callable at any time: work queued later runs on a stream of
 * that priority, after everything queued before.  For a latency-critical solver sharing
 * the GPU: a 256^2 step next to four 192^3 systems drops from about 156 to 45 us at the
 * highest level. */
int cupssgb_solver_set_stream_priority(cupssgb_solver* s, int level);
/* Steps taken so far, kernels launched so far, device bytes held. */
long long cupssgb_solver_step_count(const cupssgb_solver* s);
long long cupssgb_solver_launch_count(const cupssgb_solver* s);
long long cupssgb_solver_device_bytes(const cupssgb_solver* s);
/* The solver's CUDA stream (cudaStream_t), for callers that order their own work. */
void* cupssgb_solver_stream(const cupssgb_solver* s);
/* advance(nsteps) bracketed by CUDA events on the solver's stream; *ms = elapsed. */
int cupssgb_solver_time_advance(cupssgb_solver* s, int nsteps, double* ms);
/* Per-kernel timing of subsequent advance calls (events around every launch). */
int cupssgb_solver_set_kernel_timing(cupssgb_solver* s, int on);
/* JSON {"kind": {"launches": n, "ms": total}} of the launches timed so far; returns
 * the full length, writes at most buflen-1 chars plus a NUL. */
int cupssgb_solver_kernel_report(cupssgb_solver* s, char* buf, int buflen);

/* The update program of each non-empty phase is compiled for the system at prepare
 * time (NVRTC): straight-line code for its terms and prefactor exponents, numerical
 * values read from the parameter block.  index selects the phase program (0 = the
 * first non-empty phase).  Returns the length of the CUDA source; works without a
 * GPU.  set_generated_programs(0) switches to the table-driven update kernel. */
int cupssgb_solver_generated_source(cupssgb_solver* s, int index, char* buf, int buflen);
int cupssgb_solver_set_generated_programs(cupssgb_solver* s, int on);
/* Compiles a generated source for sm_103a without loading it (no GPU needed).
 * Returns the cubin size (> 0) or CUPSSGB_ERR_CUDA with the NVRTC log in `log`. */
int cupssgb_jit_check(const char* source, char* log, int loglen);

/* ---------------- batches ----------------
 * No counterpart in the reference (one system per evolver).  set_members(n) before
 * prepare turns a solver into a batch of n independent systems with the solver's
 * structure and grid: same fields, terms and q-monomials; each member has its own
 * prefactor values, noise amplitude, seed, state and step count.  advance() then
 * steps every active member in the same launches (replayed from CUDA graphs), and a
 * member's trajectory is the one a single solver with its values and seed gives.
 * The turnaround tile width is autotuned at prepare (tune_report).  Member m's
 * default seed is the solver's seed + m.  Member calls on a single solver: member 0. */
int cupssgb_solver_set_members(cupssgb_solver* s, int n);
int cupssgb_solver_members(const cupssgb_solver* s);
/* Values for member m; the q-monomials (exponents) must equal the solver's. */
int cupssgb_solver_set_member_term_pres(cupssgb_solver* s, int member, int field, int term, const cupssgb_pres* pres,
                                        int n);
int cupssgb_solver_set_member_implicit(cupssgb_solver* s, int member, int field, const cupssgb_pres* pres, int n);
int cupssgb_solver_set_member_noise(cupssgb_solver* s, int member, int field, const cupssgb_pres* amp);
int cupssgb_solver_set_member_seed(cupssgb_solver* s, int member, unsigned long long seed);
/* Inactive members are skipped by every launch and count no steps (slot reuse). */
int cupssgb_solver_set_member_active(cupssgb_solver* s, int member, int active);
/* Zeroes member m's fields and dealiased copies and its step count (a fresh solve). */
int cupssgb_solver_reset_member(cupssgb_solver* s, int member);
/* Steps member m has taken (synchronises the solver's stream); negative on error. */
long long cupssgb_solver_member_step(cupssgb_solver* s, int member);
/* set_real / get_real of member m (host: synchronous; device: stream-ordered). */
int cupssgb_solver_set_real_member(cupssgb_solver* s, int field, int member, const float* host_real);
int cupssgb_solver_set_real_member_device(cupssgb_solver* s, int field, int member, const float* dev_real);
int cupssgb_solver_get_real_member(cupssgb_solver* s, int field, int member, float* host_real);
int cupssgb_solver_get_real_member_device(cupssgb_solver* s, int field, int member, float* dev_real);
/* JSON {"phaseN": {"W": chosen, "ms": {candidate: ms per phase}}}; same buffer rules
 * as kernel_report. */
int cupssgb_solver_tune_report(cupssgb_solver* s, char* buf, int buflen);
/* Autotuner cache.  prepare times the launch shapes of each phase (turnaround tile
 * width, its resident-warp target, the FFT form of 512/1024-point lines, CTAs per plane
 * of the 3D xy-plane pass) and stores the winners in a text file keyed by GPU, grid,
 * batch span and update program; a later prepare with the same key reads them instead
 * of timing.  File: $CUPSSGB_TUNE_CACHE ("" or "off": no cache), else
 * $XDG_CACHE_HOME/cupss_gb300/tune_v1.txt, else $HOME/.cache/cupss_gb300/tune_v1.txt;
 * lines "cupssgb-tune-v1<TAB>key<TAB>value", appended, the last line of a key wins.
 * CUPSSGB_TUNE=0 turns tuning off.  These three calls expose the file for tools and
 * tests: the path ("" when off), the value of a key (returns its length, or
 * CUPSSGB_ERR_INVALID when absent), and appending an entry. */
int cupssgb_tune_cache_path(char* buf, int buflen);
int cupssgb_tune_cache_lookup(const char* key, char* value, int buflen);
int cupssgb_tune_cache_store(const char* key, const char* value);
/* Device bytes prepare would allocate for a batch of `members` (no GPU needed). */
long long cupssgb_solver_estimate_bytes(cupssgb_solver* s, int members);
/* 1 when all work queued on the solver's stream has finished, 0 while it runs. */
int cupssgb_solver_query(cupssgb_solver* s);

/* Fused stepping of several batched solvers of one system structure on different 1D/2D
 * grids (no counterpart in the reference): each kernel of a step is one launch over all
 * of them (the turnaround and the row pass of every grid, specialised to it, in one
 * generated kernel each), replayed from CUDA graphs.  Every member's trajectory is the
 * one its own solver would compute.  The solvers keep their buffers and their set/get
 * calls; cupssgb_multi_advance replaces cupssgb_solver_advance on them. */
typedef struct cupssgb_multi cupssgb_multi;
/* 0 when the solvers can be fused, else CUPSSGB_ERR_UNSUPPORTED with the reason in buf. */
int cupssgb_multi_check(cupssgb_solver* const* solvers, int n, char* buf, int buflen);
int cupssgb_multi_create(cupssgb_solver* const* solvers, int n, cupssgb_multi** out);
int cupssgb_multi_destroy(cupssgb_multi* m);
int cupssgb_multi_advance(cupssgb_multi* m, int nsteps);
long long cupssgb_multi_launch_count(const cupssgb_multi* m);
int cupssgb_multi_describe(const cupssgb_multi* m, char* buf, int buflen);
/* Times the fused launches against each solver stepping alone on its own stream (16 steps
 * each after 16 warm-up steps) and steps with the faster form from then on.  Zeroes every
 * field and puts every member back at step 0 afterwards, as after prepare: call it before
 * setting fields.  The choice is cached with the autotuner's.  Returns 1 (fused) or 0
 * (each solver on its own), or an error code. */
int cupssgb_multi_choose(cupssgb_multi* m);
/* Source of the fused kernels of phase 0 (non-dynamic fields) or 1 (dynamic fields) for
 * these solvers, prepared or not (no GPU needed); returns its length ("" when the phase
 * has no fields), or an error code as cupssgb_multi_check. */
int cupssgb_multi_generated_source(cupssgb_solver* const* solvers, int n, int phase, char* buf, int buflen);

/* ---------------- process helpers ---------------- */
/* Page-locked host memory for the host-buffer entry points (cudaMallocHost). */
int cupssgb_host_alloc(long long bytes, void** out);
int cupssgb_host_free(void* p);
/* Selects the CUDA device of the calling thread for subsequently created solvers. */
int cupssgb_set_device(int device);
/* Visible CUDA devices: returns their number (0 when there is none) or a negative
 * status, and writes one line per device ("<index>: <name>, <SMs> SMs, sm_<cc>, <MiB> MiB")
 * followed by a "driver <v>, runtime <v>" line into buf (the return value does not count
 * the text; buf may be NULL).  Backs check_device of the drop-in API
 * (inc/cupss/cu_utils.h:7 in the reference). */
int cupssgb_device_info(char* buf, int buflen);

/* Forward transform of one real field without any device allocation.  No counterpart
 * in the reference: it exists for callers that must not let a library allocate
 * device memory -- e.g. a host application that hands out all GPU memory from its own
 * fixed arena, where an allocation behind its back breaks its accounting or fails.
 * real_dev: sx*sy*sz floats on the device; fourier_dev: 2*sx*sy*sz floats on the
 * device, written with the unnormalised forward transform in the reference's full
 * complex layout (the same values cupssgb_solver_set_real + cupssgb_solver_get_fourier
 * give).  Both 8-byte aligned.  stream: a cudaStream_t (NULL = legacy default stream).
 * Working memory is a fixed device array inside the library (8 MiB of spectrum plus a
 * 32 KiB twiddle table) that every GPU loading the library holds until the process
 * exits; fields larger than 2^21 points are rejected with CUPSSGB_ERR_LIMIT.  The
 * first call on a device also looks up that array's device address and fills the
 * twiddle table with a synchronous copy, so make that first call before any stream
 * capture.  All calls share the one array: calls that can run at the same time on the
 * GPU (different streams, threads or processes sharing a context) race and must be
 * serialised by the caller.  Nothing in the array has to be cleared between calls:
 * each call writes every element it later reads.  The per-device set-up is done once
 * per process: a cudaDeviceReset after the first call on a device discards the twiddle
 * table, and calls on that device after such a reset are not supported. */
int cupssgb_real_to_fourier_noalloc(const float* real_dev, float* fourier_dev, int sx, int sy, int sz,
                                    void* stream);

/* ---------------- evolver level ---------------- */

/* evolver(bool with_cuda, sx[, sy[, sz]], dx[, dy[, dz]], dt, writeEvery)
 * (inc/cupss/evolver.h:31-33).  Pass sy = sz = 1 (and dy = dz = 1) for lower
 * dimensions.  with_cuda = 0 keeps the host arrays current after every step (the
 * step itself always runs on the GPU). */
int cupssgb_evolver_create(int with_cuda, int sx, int sy, int sz, float dx, float dy, float dz,
                           float dt, int write_every, cupssgb_evolver** out);
int cupssgb_evolver_destroy(cupssgb_evolver* e);
/* evolver::createField, addParameter, addEquation, addNoise, updateParameter,
 * setOutputField (src/evolver.cpp:128-196, 386-394).  Parse errors return
 * CUPSSGB_ERR_PARSE instead of exiting the process. */
int cupssgb_evolver_create_field(cupssgb_evolver* e, const char* name, int dynamic);
int cupssgb_evolver_add_parameter(cupssgb_evolver* e, const char* name, float value);
int cupssgb_evolver_add_equation(cupssgb_evolver* e, const char* equation);
int cupssgb_evolver_add_noise(cupssgb_evolver* e, const char* field, const char* amplitude);
int cupssgb_evolver_update_parameter(cupssgb_evolver* e, const char* name, float value);
int cupssgb_evolver_set_output_field(cupssgb_evolver* e, const char* field, int output);
int cupssgb_evolver_set_seed(cupssgb_evolver* e, unsigned long long seed);
/* Writes field.real_array[i].x for i < N before prepareProblem (fieldsReal). */
int cupssgb_evolver_set_real(cupssgb_evolver* e, const char* field, const float* host_real);
/* evolver::prepareProblem (src/evolver.cpp:81-126). */
int cupssgb_evolver_prepare(cupssgb_evolver* e);
/* nsteps x evolver::advanceTime, including writeOut every writeEveryNSteps. */
int cupssgb_evolver_advance(cupssgb_evolver* e, int nsteps);
/* evolver::writeOut (src/evolver.cpp:228-232). */
int cupssgb_evolver_write_out(cupssgb_evolver* e);
/* Waits until every field file queued by writeOut is written (files are written by a
 * background thread while the steps go on).  Returns 0, or CUPSSGB_ERR_INVALID with
 * the first failure (e.g. "NaN found in field phi") in cupssgb_last_error(). */
int cupssgb_evolver_flush_output(cupssgb_evolver* e);
/* Builds the system from a system file (evolver::createFromFile, src/parser.cpp:11-96):
 * sections "Fields" (name dynamic output), "Parameters" (name value) and "Equations". */
int cupssgb_evolver_create_from_file(cupssgb_evolver* e, const char* path);
/* Initial conditions written into the host array of a field (fieldsReal), before
 * prepareProblem (src/initializers.cpp:14-267; same formulas, the noise ones draw from
 * the C library's rand() seeded with time(NULL) like the reference). */
int cupssgb_evolver_initialize_uniform(cupssgb_evolver* e, const char* field, float value);
int cupssgb_evolver_initialize_uniform_noise(cupssgb_evolver* e, const char* field, float amplitude);
int cupssgb_evolver_initialize_normal_noise(cupssgb_evolver* e, const char* field, float mean, float sigma);
int cupssgb_evolver_initialize_half_system(cupssgb_evolver* e, const char* field, float value1, float value2,
                                           float interface_width, int direction);
int cupssgb_evolver_initialize_droplet(cupssgb_evolver* e, const char* field, float value_out, float value_in,
                                       float radius, float interface_width, int center_x, int center_y,
                                       int center_z);
int cupssgb_evolver_add_droplet(cupssgb_evolver* e, const char* field, float value, float radius,
                                float interface_width, int center_x, int center_y, int center_z);
int cupssgb_evolver_initialize_from_file(cupssgb_evolver* e, const char* field, const char* path, int skiprows,
                                         char delimiter);
/* Copies the host array of a field (fieldsReal[field][i].x) into host_real; no device
 * access (after prepareProblem it holds what the host wrote, not the evolved field). */
int cupssgb_evolver_get_host_real(cupssgb_evolver* e, const char* field, float* host_real);
/* Writes values (sx*sy*sz floats) as one field file in the reference's CSV format to
 * path: header "x, [y, [z, ]]<name>", one "i, [j, [k, ]]value" line per point with
 * `precision` decimals (src/field.cpp:350-402).  The dimension follows the reference's
 * rule (sy = sz = 1: 1D; sz = 1: 2D).  A NaN value stops the file with
 * CUPSSGB_ERR_INVALID ("NaN found in field <name>"). */
int cupssgb_write_field_csv(const char* path, const char* name, const float* values, int sx, int sy, int sz,
                            int precision);
/* copyAllDataToHost then field.real_array[.].x / comp_array for one field. */
int cupssgb_evolver_get_real(cupssgb_evolver* e, const char* field, float* host_real);
int cupssgb_evolver_get_fourier(cupssgb_evolver* e, const char* field, float* host_complex);
float cupssgb_evolver_get_parameter(cupssgb_evolver* e, const char* name);
int cupssgb_evolver_current_step(const cupssgb_evolver* e);
/* Parsed system as JSON: [{"name", "dynamic", "implicit": [[pre,q2n,iqx,iqy,iqz,invq]..],
 * "terms": [{"product": [names], "pres": [[..]..]}..], "noisy", "noise": [..]}..].
 * Returns the full length; writes at most buflen-1 chars plus a NUL. */
int cupssgb_evolver_describe(const cupssgb_evolver* e, char* buf, int buflen);
/* The solver behind an evolver (valid after prepare), for device-level access. */
cupssgb_solver* cupssgb_evolver_solver(cupssgb_evolver* e);
/* field::hasCB / callback (fourier = 0) or hasCBFourier / callbackFourier (fourier = 1),
 * src/field.cpp:48-86.  The callback receives the evolver, the field as float2 pairs
 * (real space: N (x, 0) values; Fourier space: N complex values, reference layout) and
 * sx, sy, sz; device pointers in GPU mode, host pointers when created with
 * with_cuda = 0.  fn = NULL removes it. */
typedef void (*cupssgb_callback)(void* evolver, float* field_pairs, int sx, int sy, int sz);
int cupssgb_evolver_set_callback(cupssgb_evolver* e, const char* field, int fourier, cupssgb_callback fn);

/* ---------------- ensemble level ----------------
 * The C++ class `ensemble` (include/cupss/ensemble.h) flattened to C: one system
 * declared with the evolver's calls, many members that differ in grid, time step,
 * seed and parameter values, grouped into batch solvers at prepare.  add_member
 * returns the member index.  advance runs every member nsteps and returns when all
 * are done.  describe: JSON list of the groups (grid, dt, members, autotuning). */
typedef struct cupssgb_ensemble cupssgb_ensemble;
int cupssgb_ensemble_create(cupssgb_ensemble** out);
int cupssgb_ensemble_destroy(cupssgb_ensemble* e);
int cupssgb_ensemble_create_field(cupssgb_ensemble* e, const char* name, int dynamic);
int cupssgb_ensemble_add_parameter(cupssgb_ensemble* e, const char* name, float value);
int cupssgb_ensemble_add_equation(cupssgb_ensemble* e, const char* equation);
int cupssgb_ensemble_add_noise(cupssgb_ensemble* e, const char* field, const char* amplitude);
int cupssgb_ensemble_add_member(cupssgb_ensemble* e, int sx, int sy, int sz, float dx, float dy, float dz, float dt,
                                unsigned long long seed);
int cupssgb_ensemble_set_member_parameter(cupssgb_ensemble* e, int member, const char* name, float value);
int cupssgb_ensemble_prepare(cupssgb_ensemble* e);
int cupssgb_ensemble_set_real(cupssgb_ensemble* e, int member, const char* field, const float* host_real);
int cupssgb_ensemble_advance(cupssgb_ensemble* e, int nsteps);
int cupssgb_ensemble_get_real(cupssgb_ensemble* e, int member, const char* field, float* host_real);
int cupssgb_ensemble_groups(const cupssgb_ensemble* e);
long long cupssgb_ensemble_device_bytes(const cupssgb_ensemble* e);
long long cupssgb_ensemble_launch_count(const cupssgb_ensemble* e);
int cupssgb_ensemble_describe(const cupssgb_ensemble* e, char* buf, int buflen);

/* ---------------- server level ----------------
 * The C++ class `server` (include/cupss/server.h) flattened to C: a scheduler thread
 * that admits submitted solves into batch-solver slots within an HBM budget, steps
 * them with continuous batching and keeps finished results in host memory.
 * Systems are declared once per add_system id.  submit copies the parameter values
 * (names[i] = values[i]) and initial fields (fields[i] -> arrays[i], sx*sy*sz floats)
 * and returns the request id (> 0).  wait returns 1 when done, 0 on timeout (timeout
 * < 0: no limit).  result: the system's output field (set_output_field, default the
 * first field).  times: seconds since the server started at submit, admission and
 * completion.  warm: creates the pool for a system, grid and time step ahead of time
 * (compilation and autotuning happen there, not in the first request). */
typedef struct cupssgb_server cupssgb_server;
int cupssgb_server_create(double hbm_budget, int max_slots, int max_chunk, cupssgb_server** out);
int cupssgb_server_destroy(cupssgb_server* s);
int cupssgb_server_add_system(cupssgb_server* s);
int cupssgb_server_create_field(cupssgb_server* s, int system, const char* name, int dynamic);
int cupssgb_server_add_parameter(cupssgb_server* s, int system, const char* name, float value);
int cupssgb_server_add_equation(cupssgb_server* s, int system, const char* equation);
int cupssgb_server_add_noise(cupssgb_server* s, int system, const char* field, const char* amplitude);
int cupssgb_server_set_output_field(cupssgb_server* s, int system, const char* field);
long long cupssgb_server_submit(cupssgb_server* s, int system, int sx, int sy, int sz, float dx, float dy, float dz,
                                float dt, long long nsteps, unsigned long long seed, int nparams,
                                const char* const* names, const float* values, int ninit,
                                const char* const* fields, const float* const* arrays);
int cupssgb_server_warm(cupssgb_server* s, int system, int sx, int sy, int sz, float dx, float dy, float dz,
                        float dt);
int cupssgb_server_wait(cupssgb_server* s, long long id, double timeout);
int cupssgb_server_result(cupssgb_server* s, long long id, float* host_out);
int cupssgb_server_times(cupssgb_server* s, long long id, double* times3);
int cupssgb_server_stats(cupssgb_server* s, char* buf, int buflen);

#ifdef __cplusplus
}
#endif

#endif /* CUPSS_GB300_H */
