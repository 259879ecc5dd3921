/*
 * fwgb.h — C ABI of the GB300 (sm_103a) FDTD engine for Fullwave 2.5 simulations.
 *
 * This library replaces the reference's engine boundary: the closed executable that
 * fullwave/solver/launcher.py:196-215 runs in a simulation directory, which reads the `.dat`
 * input set written by fullwave/solver/input_file_writer.py:105-179 and writes `genout.dat`
 * (float32, time-major [n_out, ncoordsout]) that launcher.py:243-251 loads. Here the same
 * arrays are passed in memory and the traces come back in the same layout.
 *
 * Conventions: every entry point returns an int status (FW_OK = 0); no C++ exception, abort or
 * device trap crosses this boundary. On failure, fw_last_error() describes the cause. A handle
 * is used from one host thread at a time; separate handles may run concurrently on separate
 * CUDA streams. Streams are passed as `void*` (a cudaStream_t; NULL = legacy default stream).
 */
#ifndef FWGB_H
#define FWGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FWGB_ABI_VERSION 1

#if defined(__GNUC__)
#define FWGB_API __attribute__((visibility("default")))
#else
#define FWGB_API
#endif

enum fw_status {
    FW_OK = 0,
    FW_ERR_ARGUMENT = 1,    /* a size, pointer or index is invalid */
    FW_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    FW_ERR_STATE = 3,       /* call out of order (e.g. run before fields are set) */
    FW_ERR_OOM = 4,         /* device allocation failed */
    FW_ERR_DEVICE = 5,      /* a kernel reported an error through the device status word */
    FW_ERR_UNSUPPORTED = 6  /* valid input the engine does not implement */
};

/* Scalars of the engine's file contract: nX nY nZ nT nTic modT dX dY dZ dT c0 ncoords
 * ncoordsout ncoordszero ndmap (input_file_writer.py:763-803), plus the engine variant.
 * For 2D, nz = 1 and dz is ignored. The x axis (nx) is the slowest-varying index of every map,
 * the last axis the fastest (C order, input_file_writer.py:870-881). */
typedef struct fw_desc {
    int32_t ndim;           /* 2 or 3 */
    int32_t nx, ny, nz;
    int32_t nt;             /* time steps */
    int32_t nt_ic;          /* columns of icmat: source drives steps n < nt_ic */
    int32_t mod_t;          /* record every mod_t steps (n % mod_t == 0) */
    float dx, dy, dz, dt, c0;
    int32_t ncoords;        /* source cells */
    int32_t ncoordsout;     /* sensor cells */
    int32_t ncoordszero;    /* air (zero-pressure) cells */
    int32_t ndmap;          /* tap sets in dmap, 1..65535 (a cell's index is kept in 16 bits) */
    int32_t isotropic;      /* 1: isotropic relaxation maps (fw_set_fields); 0: one set of maps
                               per derivative axis (fw_set_fields_aniso) */
    int32_t n_relax;        /* 2: the relaxation engine; 0: the exponential-attenuation engine
                               (fw_set_fields_exp, no relaxation maps) */
} fw_desc;

/* Arrays of the file contract. Maps are float32 [nx*ny*nz] C order; dcmap int32 of the same
 * shape holding 0-based tap-set indices; d float32[9*2]; dmap float32[9*2*ndmap] laid out
 * [9][2][ndmap]; icc/outc/icczero int32 [n][ndim] row-major (x, y[, z]); icmat float32
 * [ncoords][nt_ic]. `c` and `d` are accepted for contract completeness and validated but the
 * time loop reads the per-cell tap sets (dmap, dcmap), K and rho. Pointers are host memory
 * unless on_device = 1 (then device pointers on the handle's device). */
typedef struct fw_fields {
    const float *d, *dmap;
    const int32_t *dcmap;
    const float *c, *rho, *K, *beta;
    const float *kappax, *kappau;
    const float *apmlu1, *bpmlu1, *apmlx1, *bpmlx1;
    const float *apmlu2, *bpmlu2, *apmlx2, *bpmlx2;
    const int32_t *icc, *outc, *icczero;
    const float *icmat;
    int32_t on_device;
} fw_fields;

/* The anisotropic build's additional maps (same layout as the maps of fw_fields): the pressure
 * gradient along y uses kappaw, apmlw1, bpmlw1, apmlw2, bpmlw2 and along z the "v" maps; the
 * velocity divergence along y uses the "y" maps and along z the "z" maps; along x the fw_fields
 * maps ("u" for the gradient, "x" for the divergence) (input_file_writer.py:592-620).
 * The z and v maps are ignored for 2D grids. */
typedef struct fw_fields_aniso {
    const float *kappaw, *apmlw1, *bpmlw1, *apmlw2, *bpmlw2;
    const float *kappay, *apmly1, *bpmly1, *apmly2, *bpmly2;
    const float *kappav, *apmlv1, *bpmlv1, *apmlv2, *bpmlv2;
    const float *kappaz, *apmlz1, *bpmlz1, *apmlz2, *bpmlz2;
} fw_fields_aniso;

typedef struct fw_handle fw_handle;

/* Library ABI version (FWGB_ABI_VERSION). */
FWGB_API int fw_abi_version(void);

/* Create an engine for one simulation geometry on the current CUDA device.
 * Replaces: the executable's start-up that reads nX..ndmap (launcher.py:196-215). */
FWGB_API int fw_create(const fw_desc *desc, fw_handle **out);

/* Copy the medium, coefficient tables, source/sensor/air coordinates and source signals into
 * engine-owned device memory, and reset the wavefield.
 * Replaces: the executable reading d dmap dcmap c rho K beta kappa* apml* bpml* icc outc icmat
 * icczero (InputFileWriter._save_variables_into_dat_file, input_file_writer.py:563-645). */
FWGB_API int fw_set_fields(fw_handle *h, const fw_fields *f);

/* fw_set_fields for a handle created with isotropic = 0 (the anisotropic build,
 * use_isotropic_relaxation=False in the reference: medium.py:374-406). */
FWGB_API int fw_set_fields_aniso(fw_handle *h, const fw_fields *f, const fw_fields_aniso *an);

/* fw_set_fields for a handle created with n_relax = 0: the exponential-attenuation build
 * (use_exponential_attenuation=True in the reference: medium.py:560-750, input_file_writer.py:
 * 629-645). The relaxation map pointers of `f` are ignored; `a_exp` is the per-cell amplitude kept
 * per field update (same layout and on_device flag as the other maps). */
FWGB_API int fw_set_fields_exp(fw_handle *h, const fw_fields *f, const float *a_exp);

/* Replace only the source signals (a new transmit event on the same medium), float32
 * [ncoords][nt_ic]. Replaces: the is_static_map re-run that rewrites icmat.dat only
 * (input_file_writer.py:145-169). */
FWGB_API int fw_set_source_signal(fw_handle *h, const float *icmat, int32_t on_device);

/* Overwrite the source samples of steps [n0, n0 + ncols) with `cols`, float32 time-major
 * [ncols][ncoords] (row = one time step), asynchronously on `stream`; for streaming transmit
 * signals step block by step block. */
FWGB_API int fw_set_source_columns(fw_handle *h, void *stream, const float *cols, int32_t n0,
                                   int32_t ncols, int32_t on_device);

/* Record sensor groups instead of single sensors: from now on every recorded step writes
 * row[g] = sum over the sensors k with group_of_sensor[k] = g of weight[k] * p (sensors with
 * group -1 are dropped), so traces become [n_out][n_groups]. With weights 1/(sensors in the group)
 * this is the per-element averaging of Transducer.post_process_sensor_output
 * (transducer.py:807-869) done inside the time loop, without per-sensor traces. n_groups = 0
 * returns to per-sensor traces. Host arrays of ncoordsout entries. Resets the wavefield. */
FWGB_API int fw_set_sensor_groups(fw_handle *h, const int32_t *group_of_sensor,
                                  const float *weight, int32_t n_groups);

/* Full solve: reset the wavefield, run nt steps on `stream`, and copy the traces
 * [n_out][ncoordsout] (n_out = ceil(nt / mod_t)) to `out` (host memory unless
 * out_on_device = 1). Synchronises `stream` before returning when out is host memory.
 * Replaces: the executable's time loop and genout.dat (launcher.py:207-251). */
FWGB_API int fw_run(fw_handle *h, void *stream, float *out, int32_t out_on_device);

/* Zero the wavefield, memory variables, traces and step counter (asynchronous on stream). */
FWGB_API int fw_reset(fw_handle *h, void *stream);

/* Advance n_steps time steps from the current step (asynchronous on stream). The traces of
 * recorded steps accumulate in the engine's device trace buffer. */
FWGB_API int fw_advance(fw_handle *h, void *stream, int32_t n_steps);

/* Copy trace rows [row0, row0 + n_rows) to `dst` (host unless on_device = 1); asynchronous on
 * stream for device dst, synchronous for host dst. */
FWGB_API int fw_read_traces(fw_handle *h, void *stream, int32_t row0, int32_t n_rows, float *dst,
                   int32_t on_device);

/* Device pointer of the trace buffer [n_out][ncoordsout] (valid until fw_destroy). */
FWGB_API int fw_trace_buffer(fw_handle *h, float **dev_ptr);

/* Copy a wavefield component to dst as a dense C-order [nx][ny][nz] float32 array.
 * field: 0 = p, 1..3 = velocity along x, y, z (staggered +1/2 on that axis). */
FWGB_API int fw_get_field(fw_handle *h, void *stream, int32_t field, float *dst, int32_t on_device);

/* Steps taken since the last reset (host-side count of issued steps). */
FWGB_API int fw_current_step(const fw_handle *h, int32_t *step);

/* Device bytes held by the handle. */
FWGB_API int fw_device_bytes(const fw_handle *h, uint64_t *bytes);

/* Kernel family in use: 0 = direct-addressed kernels, 1 = plane/row-march kernels (TMA-staged
 * halo planes in 3D, halo rows in 2D), 2 = the persistent 2D kernel (one cooperative launch per
 * fw_advance, grid barriers between the velocity and pressure phases), 3 = the 3D plane march
 * with the point-wise state and maps staged by TMA as well (isotropic engine), 4 = the 2D tile
 * kernels (one 32 x 8 tile per block, every operand staged by TMA; every cell physics). 3D handles
 * use 3
 * (isotropic; 1 with FWGB_STREAM3D=0) or 1 (anisotropic, exponential) unless the environment
 * variable FWGB_VARIANT=direct was set when the handle was created. 2D handles
 * start on 0 and the first fw_advance from step 0 autotunes the kernel shape (direct, a march
 * block of TY columns x XC rows, persistent, or TMA tiles), timing each shape for a few dozen
 * steps on the
 * handle itself and resetting it after each trial; the choice is cached per device, grid size and
 * physics. FWGB_AUTOTUNE=0 disables the trials, FWGB_VARIANT=direct|march or
 * FWGB_SHAPE2D=<index 0-7> fixes the shape at creation (groups: 0-5; the single-simulation shapes
 * 6-7 give a group the direct kernels). Every shape gives bit-identical results.
 * No counterpart in the reference (one CUDA kernel family). */
FWGB_API int fw_kernel_variant(const fw_handle *h, int32_t *variant);

/* Cells per block of the kernels in use, along (x, y, z) (z = 1 in 2D). No counterpart in the
 * reference. */
FWGB_API int fw_block_tile(const fw_handle *h, int32_t tile[3]);

/* Copy n_rows x-rows (depth rows) of every state field (p, velocities, memory variables) from
 * src rows [src_row0, src_row0 + n_rows) to dst rows [dst_row0, ...), asynchronously on stream.
 * The two grids must have the same cross-section (ny, nz). This is the halo exchange of a depth
 * slab decomposition (fullwave25_gb300.slabs): the reference splits depth into per-GPU slabs
 * inside its executables (README.md:249-261); here slabs of one simulation exchange their
 * overlap rows every step through this call. */
FWGB_API int fw_copy_state_rows(fw_handle *dst, int32_t dst_row0, const fw_handle *src,
                                int32_t src_row0, int32_t n_rows, void *stream);

/* Failure-detection self-test: runs a kernel that waits on an mbarrier nothing completes and a
 * one-block kernel at a grid barrier that counts two blocks; each wait gives up after its limit
 * (0.5 s, 1 s) and records it in a status word instead of hanging. status_out[0] = the mbarrier
 * kernel's status (bit 0x1 expected), status_out[1] = the grid-barrier kernel's (bit 0x4
 * expected). Takes about 1.5 s. No counterpart in the reference. */
FWGB_API int fw_selftest_waits(int32_t status_out[2]);

/* Kernel launches issued per time step (for launch accounting). */
FWGB_API int fw_launches_per_step(const fw_handle *h, int32_t *n);

/* Release all device memory of the handle. */
FWGB_API int fw_destroy(fw_handle *h);

/* Gradient of the sensor-trace misfit J = 1/2 sum ||traces - observed||^2 (2D and 3D; isotropic
 * or anisotropic relaxation, or exponential-attenuation engine; linear or with beta; individual
 * sensor traces: no sensor groups), with respect to the engine's coefficient maps, by the
 * discrete adjoint of the time step. No counterpart in the reference (it has no gradient
 * computation).
 * fw_adjoint_forward: run the full forward solve from rest, keeping a checkpoint of the wavefield
 * every `checkpoint_every` steps (device memory: nt / checkpoint_every + 2 (checkpoint_every + 1)
 * wavefield copies: the checkpoints and two state stores; one store in 3D, or with
 * FWGB_ADJ_OVERLAP=0 at this call); the traces are then available from fw_read_traces. */
FWGB_API int fw_adjoint_forward(fw_handle *h, void *stream, int32_t checkpoint_every);

/* Reverse pass: recompute each segment from its checkpoint and run the adjoint step backwards,
 * accumulating the gradient: each step's contributions are formed in FP32 (the precision of the
 * adjoint fields) into per-segment FP32 partial sums that are added into FP64 time sums at the
 * end of every segment (FWGB_ADJ_F64_STEPS=1: every step's contributions in FP64 instead).
 * 2D: each reverse step is two launches whose operands are staged in shared memory by TMA
 * (FWGB_ADJ_TMA=0: the same arithmetic with the operands loaded by the threads). With two state
 * stores, the next segment is recomputed into one on a second (internal) stream while the current
 * segment is reversed from the other on `stream`; the gradient is bitwise the same as one segment
 * after another. 3D: the segment is recomputed in place (state copies into the store), then each
 * reverse step is four launches with the operands loaded by the threads.
 * `residual` = traces - observed, device float32 [n_out][ncoordsout]. `grad_out`: device FP64
 * [12][nx][ny] (3D: [12][nx][ny][nz]) in the order dt/rho, dt*K, 1/kappau, 1/kappax, au1, bu1,
 * au2, bu2, ax1, bx1, ax2, bx2 (ghost cells zero); the exponential-attenuation engine fills dt/rho,
 * dt*K and, in the au1 slot, a_exp, and leaves the other slots zero; the anisotropic engine
 * returns [2 + 10 ndim][...]: dt/rho, dt*K, then for each derivative axis 1/kappa, a1, b1, a2, b2
 * of its pressure-gradient maps (u, w, v), then the same of its velocity-divergence maps
 * (x, y, z). When beta is not zero everywhere one more array follows: the gradient with
 * respect to 2 dt beta. Those engines' reverse step, and any reverse step with beta, is four
 * thread-load launches in 2D and 3D. The wavefield left in the handle afterwards is the first segment's
 * recomputation. Returns after the stream has finished the pass (FW_ERR_DEVICE if a kernel
 * reported a timed-out wait). */
FWGB_API int fw_adjoint_backward(fw_handle *h, void *stream, const float *residual,
                                 double *grad_out);

/* A group runs many independent 2D simulations together: every time step is one velocity
 * launch and one pressure launch over a device work list of (simulation, tile) pairs, so small
 * simulations share the GPU instead of each leaving it mostly idle; blocks of 64 steps are
 * captured into CUDA graphs. Members keep their own memory, sources, sensors and nt (a member
 * stops stepping at its nt; its tiles leave the work list). No counterpart in the reference,
 * which runs one executable per simulation (fullwave/solver/launcher.py:196-215). */
typedef struct fw_group fw_group;

/* Build a group over 2D handles whose fields are set (the handles must outlive the group). */
FWGB_API int fw_group_create(fw_handle *const *handles, int32_t n, fw_group **out);

/* Reset every member and run each for its own nt steps (asynchronous on stream); afterwards
 * read each member's traces with fw_read_traces. The whole run is captured once into one CUDA
 * graph (every step's two launches over the shrinking prefix of active members) and replayed by
 * later runs while the members and the kernel shape stay the same (FWGB_GROUP_RUN_GRAPH=0: blocks
 * of 64-step graphs as fw_group_advance issues them; FWGB_GROUP_PERSISTENT=1: the whole run as
 * one persistent cooperative launch with grid barriers between the phases, row-march shapes,
 * bitwise the same traces). Errors: fw_last_error(NULL). */
FWGB_API int fw_group_run(fw_group *g, void *stream);

/* Replace the member list (members may be at different steps; continuous batching admits new
 * simulations and retires finished ones between calls to fw_group_advance). */
FWGB_API int fw_group_set_members(fw_group *g, fw_handle *const *handles, int32_t n);

/* Advance every member by up to n_steps time steps, each stopping at its own nt
 * (asynchronous on stream). */
FWGB_API int fw_group_advance(fw_group *g, void *stream, int32_t n_steps);

/* Release the group (not its members). */
/* Cells per block of the group's kernels along (x, y, z). The group starts on the 128 x 32 row
 * march (or the shape FWGB_VARIANT / FWGB_SHAPE2D fix at creation); the first fw_group_run
 * times every 2D kernel shape on the group itself (members reset after each trial) and keeps the
 * fastest. FWGB_AUTOTUNE=0 disables the trials. No counterpart in the reference. */
FWGB_API int fw_group_block_tile(const fw_group *g, int32_t tile[3]);

FWGB_API int fw_group_destroy(fw_group *g);

/* Bytes of the file-scope device array in which fw_run_noalloc keeps everything it needs besides
 * the caller's inputs and outputs (48 MiB): 66 bytes per grid cell (11 state fields, 5 derived
 * coefficient maps, a 16-bit tap index) plus 48 bytes per tap set and one byte per source, so 2D
 * grids up to about 760,000 cells (e.g. the 944 x 688 PML-extended plain 2D workload). */
#define FWGB_NOALLOC_SCRATCH_BYTES (48u * 1024u * 1024u)

/* Full 2D forward solve that allocates nothing. This entry point has no counterpart in the
 * reference; it exists for callers that cannot call cudaMalloc while they run: applications whose
 * device memory comes only from their own pool, processes that must not grow their device
 * footprint after start-up, or code that only holds device buffers handed to it. Inputs
 * (`f`, with on_device = 1: device pointers) and the output traces (device memory,
 * [n_out][ncoordsout]) are the caller's; the wavefield, memory variables, derived maps and tap
 * table live in one file-scope device array of FWGB_NOALLOC_SCRATCH_BYTES that every GPU which
 * loads this library holds until the process exits. Grids that need more than that are rejected
 * with FW_ERR_ARGUMENT; 3D grids with FW_ERR_UNSUPPORTED.
 * Before stepping, every source, sensor and air coordinate and every dcmap entry is checked on the
 * device against the grid; the call waits for that check (it synchronises `stream` once) and
 * returns FW_ERR_ARGUMENT, naming the first offending entry, without running any time step and
 * without writing `traces`, if one lies outside. A cell listed twice as a source is driven by its
 * last entry. After the check the solve is queued asynchronously on `stream`; its traces equal
 * those of fw_create + fw_set_fields + fw_run bit for bit.
 * Each call clears the parts of the array it uses that must start at zero; the array keeps the
 * last call's contents afterwards. All calls share the one array, so calls that overlap on the GPU
 * (other streams, other host threads) race: serialise them. Each call looks the array's device
 * address up (cudaGetSymbolAddress) with the calling thread's current device; the first call on a
 * device also loads this library's device code there, so make that first call before any stream
 * capture. Errors are reported by fw_last_error(NULL). */
FWGB_API int fw_run_noalloc(const fw_desc *desc, const fw_fields *f, void *stream, float *traces);

/* Description of the last failure on this handle (or of the last failed fw_create when
 * h == NULL). Never NULL. */
FWGB_API const char *fw_last_error(const fw_handle *h);

#ifdef __cplusplus
}
#endif

#endif /* FWGB_H */
