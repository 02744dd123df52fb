/*
 * everett_cuda.h -- C ABI of the GB300 statevector engine.
 *
 * This is the drop-in boundary for everett's dense statevector run path
 * (`StateVectorBackend::run(&Circuit) -> Result<Execution>`,
 * src/backend/statevector.rs:68-90).  Every entry point takes plain pointers
 * and sizes, returns 0 (EV_OK) or an EV_ERR_* code, and records a message
 * readable through ev_last_error() on the calling thread.
 *
 * Conventions
 *   - Qubit 0 is the least-significant bit of a basis index
 *     (src/qubit.rs:9-14).
 *   - Complex numbers travel as interleaved f64 pairs [re, im], the layout of
 *     the reference's #[repr(C)] Complex64 (src/complex.rs:22-29).
 *   - A 1-qubit matrix is 4 complex entries row-major [m00, m01, m10, m11]
 *     (src/gate.rs:21-25) = 8 doubles.  A 2-qubit matrix is 16 complex entries
 *     row-major in the basis |q_a q_b> with a the more significant operand
 *     (src/gate.rs:27-35) = 32 doubles.
 *   - The library owns device memory; callers own every host buffer.
 *   - A state handle is used from one host thread at a time.  Each state owns
 *     its own CUDA stream, so work on different states may overlap.
 */
#ifndef EVERETT_CUDA_H
#define EVERETT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---------------------------------------------------------
 * The first four mirror the variants of everett::Error that the statevector
 * path can raise (src/error.rs:10-53); the rest are device-side conditions
 * the CPU crate cannot meet. */
enum {
  EV_OK = 0,
  EV_ERR_QUBIT_OUT_OF_RANGE = 1,         /* Error::QubitOutOfRange        */
  EV_ERR_CLASSICAL_BIT_OUT_OF_RANGE = 2, /* Error::ClassicalBitOutOfRange */
  EV_ERR_DUPLICATE_QUBIT = 3,            /* Error::DuplicateQubit         */
  EV_ERR_DIMENSION_MISMATCH = 4,         /* Error::DimensionMismatch      */
  EV_ERR_NON_CLIFFORD = 5,               /* Error::NonClifford            */
  EV_ERR_QASM = 6,                       /* Error::Qasm (line:col in the message) */
  EV_ERR_INVALID_ARGUMENT = 16, /* null pointer, bad dtype, malformed op list */
  EV_ERR_OOM = 17,              /* device allocation refused              */
  EV_ERR_CUDA = 18,             /* a CUDA runtime call failed             */
  EV_ERR_TIMEOUT = 19,          /* a bounded device wait gave up          */
  EV_ERR_ADMISSION = 20,        /* serve: request can never fit in HBM    */
  EV_ERR_CANCELLED = 21         /* serve: request cancelled before it ran */
};

/* amplitude storage types */
enum { EV_C128 = 0, EV_C64 = 1 };

/* ---- operations ----------------------------------------------------------
 * One ev_op per everett::Op variant (src/op.rs:14-58).  IfClassic
 * (`Op::IfClassic { bit, then: Box<Op> }`) is encoded in prefix form: an
 * EV_OP_IF record with q0 = the classical bit is followed by the record(s)
 * of its body, which may itself be another EV_OP_IF. */
enum {
  EV_OP_APPLY1 = 1,     /* gate m[0..8)  on target q0                      */
  EV_OP_APPLY2 = 2,     /* gate m[0..32) on operands a = q0, b = q1        */
  EV_OP_CONTROLLED = 3, /* gate m[0..8) on target q0, controls in the pool */
  EV_OP_MEASURE = 4,    /* measure qubit q0 into classical bit q1          */
  EV_OP_IF = 5          /* run the next op only if classical bit q0 is set */
};

typedef struct ev_op {
  uint32_t kind;     /* EV_OP_*                                            */
  uint32_t nctrl;    /* EV_OP_CONTROLLED: number of controls               */
  uint64_t ctrl_off; /* EV_OP_CONTROLLED: index of first control in pool   */
  uint64_t q0;
  uint64_t q1;
  double m[32];      /* interleaved re,im; 8 used by 1-qubit gates         */
} ev_op;

/* A circuit: register sizes, the op list and the pool of control indices
 * (`Circuit { ops, num_qubits, num_classical }`, src/circuit.rs:26-30). */
typedef struct ev_circuit {
  uint64_t num_qubits;
  uint64_t num_classical;
  const ev_op* ops;
  uint64_t nops;
  const uint64_t* ctrl_pool;
  uint64_t pool_len;
} ev_circuit;

/* Execution options of the run loop. */
enum {
  EV_MODE_EXACT = 0, /* one kernel per op, the reference's arithmetic order */
  EV_MODE_TILED = 1, /* runs of ops applied to shared-memory tiles, one HBM
                        pass per run; same per-amplitude arithmetic        */
  EV_MODE_FUSED = 2  /* runs of ops fused on the host (f64) into dense
                        k-qubit unitaries, one HBM pass each; complex64
                        with the variants below but EV_FUSED_OZAKI and
                        EV_FUSED_OZAKI6, the complex128 ones              */
};
/* Arithmetic of a fused k-qubit unitary (EV_MODE_FUSED). */
enum {
  EV_FUSED_TF32X3 = 0, /* tensor cores, split TF32 products, f32 accumulate */
  EV_FUSED_BF16X3 = 1, /* tensor cores, split BF16 products, f32 accumulate */
  EV_FUSED_FP32 = 2,   /* CUDA cores, f32 complex multiply-add              */
  EV_FUSED_OZAKI = 3,  /* complex128: tensor cores, each f64 as seven 8-bit
                          digits in FP16 (per-row / per-column scale), digit
                          products summed exactly in f32, recombined in
                          int64 (the Ozaki scheme); k = 5; a NaN or an
                          infinity in the state makes the run return
                          EV_ERR_INVALID_ARGUMENT                          */
  EV_FUSED_OZAKI6 = 4  /* complex128: the same with six digits (47 bits per
                          value below its row's or column's maximum): fewer
                          MMAs and digit slices, ~7e-14 of a row's largest
                          value per pass instead of ~3e-16                */
};
typedef struct ev_run_options {
  int32_t dtype;     /* EV_C128 or EV_C64                                  */
  int32_t mode;      /* EV_MODE_*                                          */
  int32_t tile_bits; /* tiled: qubits per tile; fused: qubits per unitary
                        (0 = default)                                      */
  int32_t variant;   /* fused: EV_FUSED_*                                  */
} ev_run_options;

typedef struct ev_state ev_state;

/* ---- library ---------------------------------------------------------- */

/* Message of the last failing call on this thread ("" if none). */
const char* ev_last_error(void);
/* Version string of the library. */
const char* ev_version(void);
/* Number of CUDA devices the library can see (0 on a host without a GPU). */
int ev_device_count(int* out);

/* ---- state storage (src/state.rs:24-90) ------------------------------- */

/* |0...0> on n qubits (State::zero, src/state.rs:39-44).  EV_ERR_OOM if the
 * 2^n x 16 (or 8) byte buffer does not fit. */
int ev_state_create(uint64_t n, int32_t dtype, ev_state** out);
int ev_state_destroy(ev_state* s);
int ev_state_num_qubits(const ev_state* s, uint64_t* out);
int ev_state_dtype(const ev_state* s, int32_t* out);
/* Reset to |0...0>. */
int ev_state_set_zero(ev_state* s);
/* Copy 2^n complex amplitudes (interleaved f64) into / out of the state
 * (State::from_amplitudes / amplitudes, src/state.rs:51-90).  len is the
 * number of complex amplitudes; EV_ERR_DIMENSION_MISMATCH unless len == 2^n.
 * complex64 states convert on the device. */
int ev_state_upload(ev_state* s, const double* amps, uint64_t len);
int ev_state_download(const ev_state* s, double* amps, uint64_t len);
/* Wait until all work queued on the state's stream has finished. */
int ev_state_synchronize(const ev_state* s);

/* ---- gate kernels (src/kernel.rs:76, :192, :299) ------------------------ */

/* Single-qubit gate on qubit k (kernel::apply_1q). */
int ev_apply_1q(ev_state* s, uint64_t k, const double m[8]);
/* Two-qubit gate on operands a (more significant) and b (kernel::apply_2q).
 * CNOT, CZ and SWAP are recognised by exact matrix equality, as in
 * src/kernel.rs:201-212. */
int ev_apply_2q(ev_state* s, uint64_t a, uint64_t b, const double m[32]);
/* Single-qubit gate on target, applied where every control is set
 * (kernel::apply_controlled_1q). */
int ev_apply_controlled_1q(ev_state* s, const uint64_t* controls,
                           uint64_t ncontrols, uint64_t target,
                           const double m[8]);

/* ---- measurement (src/measure.rs:15-51) -------------------------------- */

/* Measure qubit k with the caller's uniform u in [0,1): outcome = u < p1,
 * then collapse and rescale by 1/sqrt(surviving). */
int ev_measure_qubit(ev_state* s, uint64_t k, double u, int32_t* outcome);

/* No counterpart in the reference.  The same measurement on a complex128
 * statevector in a device buffer the caller owns (2^n interleaved re,im
 * doubles), for callers that cannot call cudaMalloc: one whose device memory
 * is all handed out by its own allocator, or one that cannot accept the
 * device-wide synchronisation of an allocation.  It allocates nothing: its
 * scratch is a fixed ~64 KiB array (2048 reduction blocks) in the library's
 * device memory, held on every GPU that loads the library until the process
 * exits.  n <= 40 (EV_ERR_INVALID_ARGUMENT beyond).  The buffer must be
 * 16-byte aligned device (or managed) memory of the current device holding
 * 2^n amplitudes; anything else is EV_ERR_INVALID_ARGUMENT before any launch.
 * stream may be NULL (legacy default stream).  The call synchronises that
 * stream and returns after the measurement has completed, so it cannot be
 * recorded into a CUDA graph (not during a stream capture either).  Its
 * device address of the scratch array is resolved per CUDA context.  Calls
 * share the array: calls that overlap on the GPU race, ordered calls do not. */
int ev_measure_qubit_noalloc(double* amps, uint64_t n, uint64_t k, double u,
                             void* stream, int32_t* outcome);

/* ---- observables (src/state.rs:94-185) --------------------------------- */

int ev_norm_sqr(const ev_state* s, double* out);
int ev_normalize(ev_state* s);
int ev_probability(const ev_state* s, uint64_t basis, double* out);
/* One amplitude as [re, im] (State::amplitudes()[basis], src/state.rs:81-83). */
int ev_amplitude(const ev_state* s, uint64_t basis, double out[2]);
/* <other|self> as [re, im]; the two states may differ in amplitude type
 * (both are promoted to f64). */
int ev_overlap(const ev_state* self, const ev_state* other, double out[2]);
int ev_fidelity(const ev_state* self, const ev_state* other, double* out);
/* Marginal distribution of the low m qubits (m <= 28): out[c] (2^m
 * doubles) = sum over the other qubits of |a[t * 2^m + c]|^2, summed in
 * basis order as most_probable_phase does (phase_estimation.rs:97-110). */
int ev_marginal_low(const ev_state* s, uint64_t m, double* out);
/* [<X>, <Y>, <Z>] of one qubit (State::bloch_vector). */
int ev_bloch_vector(const ev_state* s, uint64_t qubit, double out[3]);

/* ---- circuits (src/circuit.rs:245-306, src/backend/mod.rs:43-72) ------- */

/* Circuit::validate: the first error in op order, with the reference's
 * check order inside each op. */
int ev_validate(const ev_circuit* c);
/* StateVectorBackend::run_seeded: validate, start from |0...0>, seed the
 * measurement Rng (xoshiro256++ via SplitMix64, src/rng.rs:18-58) and walk
 * the ops.  On success *state_out is a new device-resident state owned by
 * the caller and classical_out[0..num_classical) holds the register
 * (0/1 bytes).  opts may be NULL (complex128, tiled mode: bit-identical to
 * the exact mode and faster). */
int ev_run_seeded(const ev_circuit* c, uint64_t seed, const ev_run_options* opts,
                  ev_state** state_out, uint8_t* classical_out);

/* The same run on an existing state of matching size and type: the state is
 * reset to |0...0> first, so a caller can reuse one device buffer for many
 * runs (the serving loop and the benchmark do). */
int ev_state_run(ev_state* s, const ev_circuit* c, uint64_t seed,
                 const ev_run_options* opts, uint8_t* classical_out);
/* drive (src/backend/mod.rs:43-72): the same op walk applied to the state as
 * it stands, without the reset -- what a Backend does with a circuit's ops
 * on its current state.  The classical register starts at all-zero. */
int ev_state_drive(ev_state* s, const ev_circuit* c, uint64_t seed,
                   const ev_run_options* opts, uint8_t* classical_out);

/* <psi|P|psi> for Pauli strings (PauliString::expectation,
 * src/backend/stabilizer.rs:79-125): term t is (-1)^negative[t] times the
 * product over qubits q of X (bit q set in x_masks[t] only), Z (z_masks[t]
 * only) or Y (both).  negative may be NULL (all +).  Terms sharing an X mask
 * and the parity of their Y count are evaluated in one pass over the state
 * (up to 8 per pass).  EV_ERR_QUBIT_OUT_OF_RANGE if a mask names a qubit
 * outside the register. */
int ev_pauli_expectation(const ev_state* s, const uint64_t* x_masks, const uint64_t* z_masks,
                         const uint8_t* negative, uint64_t count, double* out);

/* ---- shot sampling (no reference counterpart) ---------------------------
 * Shot j measures qubits 0..n-1 in order, each exactly as measure_qubit
 * would on the collapsed copy, with the uniforms of Rng::seed_from_u64(seed)
 * taken n per shot, shots in order.  Bit q of out[j] is qubit q's outcome.
 * The state is not modified.  n <= 63. */
int ev_sample(ev_state* s, uint64_t seed, uint64_t shots, uint64_t* out);

/* ---- batched runs (no reference counterpart) ------------------------------
 * Many independent circuits of uneven qubit counts in one persistent launch
 * over a device work queue.  Each circuit runs from |0...0> and reports
 * <Z_0> (bloch_vector(0)[2] of the final state, normalised) and `shots`
 * full-register shots drawn exactly as ev_sample draws them with its own
 * seed.  A circuit may also measure (EV_OP_MEASURE) and gate ops on its
 * classical bits (EV_OP_IF), as drive does (src/backend/mod.rs:43-72), with
 * the uniforms of Rng::seed_from_u64(run_seed); such a circuit must have at
 * most as many qubits as the tile size (it runs whole in one CTA) and at
 * most 64 classical bits, else EV_ERR_INVALID_ARGUMENT.  Output pointers
 * may be NULL. */
typedef struct ev_batch_circuit {
  ev_circuit circuit;
  uint64_t seed;       /* Rng seed of the shot stream                      */
  uint64_t shots;
  uint64_t* shots_out; /* [shots]                                          */
  double* expz_out;    /* <Z_0>                                            */
  double* amps_out;    /* final state, 2^n interleaved f64 (test hook)     */
  uint64_t run_seed;   /* Rng seed of the mid-circuit measurements, as
                          ev_run_seeded's seed                            */
  uint8_t* classical_out; /* [num_classical] 0/1 bytes, or NULL           */
} ev_batch_circuit;

typedef struct ev_batch_options {
  int32_t dtype;     /* EV_C64 (default) or EV_C128                        */
  int32_t tile_bits; /* qubits per shared-memory tile; 0 = autotuned       */
  int32_t threads;   /* threads per resident CTA (256 / 512); 0 = autotuned */
  int32_t autotune;  /* 1: time candidates when no cached choice exists   */
  int32_t test_stall; /* test hook: 1 adds a queue item whose dependency is
                         never met, so a bounded device wait runs out and
                         the call returns EV_ERR_TIMEOUT                  */
  int32_t reserved;
} ev_batch_options;

typedef struct ev_batch_stats {
  double device_ms;  /* persistent launch + uniform generation            */
  double host_ms;    /* planning, copies, result scatter                  */
  uint64_t items;    /* work-queue items                                   */
  uint64_t launches; /* kernels launched                                   */
  int32_t tile_bits; /* configuration used                                 */
  int32_t threads;
  int32_t from_cache; /* 1 if the configuration came from the tuning cache */
  int32_t reserved;
} ev_batch_stats;

int ev_batch_run(const ev_batch_circuit* items, uint64_t count, const ev_batch_options* opts,
                 ev_batch_stats* stats);

/* ---- density matrices (src/density.rs, src/noise.rs,
 *      src/backend/density_matrix.rs) ------------------------------------------
 * A 2^n x 2^n complex128 matrix resident in HBM, row-major (element (i, j) at
 * i * 2^n + j).  Gates act as rho -> U rho U^dagger, channels as
 * rho -> sum_k K_k rho K_k^dagger, with the reference's operation order, so
 * results equal DensityMatrixBackend's bit for bit (signed zeros aside) until
 * a measurement, whose probability sums agree to rounding.
 *
 * NoiseModel (noise.rs): after_1q follows every 1-qubit gate and, on the
 * target then each control, every controlled gate; after_2q follows every
 * 2-qubit gate on operand a, then b; readout_error flips a reported
 * measurement bit with that probability (one more uniform per measurement
 * when it is > 0).  A channel with nops == 0 is absent. */
#define EV_MAX_KRAUS 16
typedef struct ev_channel {
  uint32_t nops;                  /* Kraus operators in k[0 .. nops)             */
  uint32_t reserved;
  double k[EV_MAX_KRAUS][8];      /* each a row-major 2x2, interleaved re, im     */
} ev_channel;

typedef struct ev_noise_model {
  ev_channel after_1q;
  ev_channel after_2q;
  double readout_error;
} ev_noise_model;

typedef struct ev_dm ev_dm;

/* |0...0><0...0| (DensityMatrix::zero, density.rs:46-58); EV_ERR_OOM when
 * the 4^n elements cannot be stored. */
int ev_dm_create(uint64_t n, ev_dm** out);
int ev_dm_destroy(ev_dm* d);
int ev_dm_num_qubits(const ev_dm* d, uint64_t* out);
/* |psi><psi| (DensityMatrix::from_statevector, density.rs:66-82);
 * EV_ERR_DIMENSION_MISMATCH unless len is a power of two. */
int ev_dm_from_amplitudes(const double* amps, uint64_t len, ev_dm** out);
int ev_dm_download(const ev_dm* d, double* data, uint64_t len); /* len = 4^n elements */
int ev_dm_get(const ev_dm* d, uint64_t i, uint64_t j, double out[2]);
int ev_dm_trace(const ev_dm* d, double* out);
int ev_dm_purity(const ev_dm* d, double* out);
int ev_dm_probability(const ev_dm* d, uint64_t basis, double* out);
/* Tr(P rho) for P one of 'I', 'X', 'Y', 'Z' on one qubit (density.rs:236-266). */
int ev_dm_expectation_pauli(const ev_dm* d, uint64_t qubit, char observable, double* out);
/* The reduced 2x2 matrix of one qubit, [r00, r01, r10, r11] interleaved
 * (density.rs:275-295). */
int ev_dm_partial_trace_1q(const ev_dm* d, uint64_t qubit, double out[8]);
/* DensityMatrixBackend::run_with_noise_seeded (density_matrix.rs:60-79):
 * validate, |0..0><0..0|, Rng::seed_from_u64(seed), walk the ops; noise may
 * be NULL (ideal). */
int ev_dm_run(const ev_circuit* c, const ev_noise_model* noise, uint64_t seed, ev_dm** out,
              uint8_t* classical_out);

/* ---- stabilizer tableau (src/backend/stabilizer.rs) -------------------------
 * StabilizerBackend::run_seeded: a Clifford circuit on an Aaronson-Gottesman
 * tableau held bit-packed in HBM.  Gates are recognised up to global phase as
 * the reference does (H, S, S^dagger, X, Y, Z; CNOT, CZ, SWAP; singly
 * controlled X and Z); any other gate makes the run fail with
 * EV_ERR_NON_CLIFFORD after the op walk, as the reference's poisoned backend
 * does.  A random measurement outcome is next_u64() & 1 of the seeded Rng. */
typedef struct ev_stab ev_stab;

int ev_stab_run(const ev_circuit* c, uint64_t seed, ev_stab** out, uint8_t* classical_out);
int ev_stab_num_qubits(const ev_stab* t, uint64_t* out);
/* The n stabilizer generators (StabilizerExecution::generators): x and z are
 * n x n bytes, row i = generator i, column q = qubit q; neg[i] = 1 for sign -1. */
int ev_stab_generators(const ev_stab* t, uint8_t* x, uint8_t* z, uint8_t* neg);
int ev_stab_destroy(ev_stab* t);

/* ---- prepared runs (no reference counterpart) ------------------------------
 * A circuit planned once for one state and recorded as a CUDA graph.  Each
 * launch replays the whole run with one graph launch: reset to |0...0>, the
 * gate, tile or fused passes, device-side measurement and classical control,
 * and the final renormalisation of complex64 runs.  A launch gives exactly
 * what ev_state_run gives for the same circuit, options and seed.  The
 * circuit may be freed after ev_prepare; the state must outlive the prepared
 * run, and no other call may use the state while a launch is in flight. */
typedef struct ev_prepared ev_prepared;

int ev_prepare(ev_state* s, const ev_circuit* c, const ev_run_options* opts, ev_prepared** out);
/* Runs the prepared circuit with the measurement stream seeded by seed and
 * copies the classical register (num_classical bytes, 0/1) to classical_out. */
int ev_prepared_launch(ev_prepared* p, uint64_t seed, uint8_t* classical_out);
int ev_prepared_kernels(const ev_prepared* p, uint64_t* out); /* kernels per launch */
int ev_prepared_destroy(ev_prepared* p);

/* ---- OpenQASM 3 (src/qasm/mod.rs, parse.rs, emit.rs) -------------------------
 * ev_qasm_parse replaces Circuit::from_qasm (src/circuit.rs:324, parse.rs:813):
 * the same subset, circuit and errors.  On EV_ERR_QASM the message reads
 * "OpenQASM 3 error at L:C: ..." and err_line / err_col (either may be NULL)
 * receive L and C (0 when the reference reports no position).  The program
 * owns its op records; ev_program_circuit gives a view valid until
 * ev_program_free.  ev_qasm_emit replaces Circuit::to_qasm (emit.rs:17):
 * *len receives the text's length; with buf non-NULL the text and a NUL are
 * written if cap allows (EV_ERR_INVALID_ARGUMENT otherwise).  Gates without
 * a stdgates.inc name and nested IfClassic are EV_ERR_QASM. */
typedef struct ev_program ev_program;

int ev_qasm_parse(const char* src, uint64_t len, ev_program** out, uint64_t* err_line,
                  uint64_t* err_col);
int ev_program_circuit(const ev_program* p, ev_circuit* out);
int ev_program_free(ev_program* p);
int ev_qasm_emit(const ev_circuit* c, char* buf, uint64_t cap, uint64_t* len);

/* ---- serving (no reference counterpart) ------------------------------------
 * A continuous-batching request loop.  Requests are admitted in arrival
 * order while the state memory of admitted requests (2^n x 16 or 8 bytes)
 * stays within the budget; admitted requests run concurrently on separate
 * streams, and small requests admitted together share one batched launch.
 * Mid-circuit measurement and classical control stay on the device, in
 * batched launches as in single-request runs.
 * A request's result does not depend on what else is in flight. */
typedef struct ev_server ev_server;

typedef struct ev_server_options {
  int32_t dtype;        /* EV_C64 (default) or EV_C128                     */
  int32_t workers;      /* requests (or batches) in flight; 0 = 8          */
  int32_t mode;         /* EV_MODE_* of single-request runs                */
  int32_t variant;      /* EV_FUSED_* when mode is EV_MODE_FUSED           */
  uint64_t hbm_budget;  /* state bytes admitted at once; 0 = 80% of free   */
  int32_t batch_small;  /* 1: requests of <= batch_qubits qubits and <= 64
                           classical bits run through batched launches     */
  int32_t batch_qubits; /* 0 = 13 (complex64) / 12 (complex128)            */
  int32_t start_paused; /* 1: admit nothing until ev_server_resume         */
  int32_t reserved;
} ev_server_options;

typedef struct ev_server_result {
  uint64_t id;
  int32_t status;        /* EV_OK, EV_ERR_ADMISSION, EV_ERR_CANCELLED, ... */
  int32_t num_classical;
  uint64_t shots;        /* shots written to the submit-time buffer        */
  double queue_ms;       /* submit -> admitted                             */
  double latency_ms;     /* submit -> result ready                         */
  uint8_t classical[64]; /* first 64 classical bits                        */
} ev_server_result;

typedef struct ev_server_stats {
  uint64_t submitted, admitted, completed, failed, refused, cancelled;
  uint64_t running, pending, batched_launches, batched_requests;
  uint64_t reserved_bytes, budget_bytes;
} ev_server_stats;

int ev_server_create(const ev_server_options* opts, ev_server** out);
/* Copies the circuit; shots_out (shots entries) must stay valid until the
 * request's result has been polled.  A request whose state can never fit the
 * budget completes at once with EV_ERR_ADMISSION. */
int ev_server_submit(ev_server* s, const ev_circuit* c, uint64_t seed, uint64_t shots,
                     uint64_t* shots_out, uint64_t* id);
/* Submits OpenQASM 3 text (parsed at once with ev_qasm_parse's rules; a
 * parse error is returned here as EV_ERR_QASM and nothing is queued). */
int ev_server_submit_qasm(ev_server* s, const char* src, uint64_t len, uint64_t seed,
                          uint64_t shots, uint64_t* shots_out, uint64_t* id);
/* Cancels a request that has not been admitted yet. */
int ev_server_cancel(ev_server* s, uint64_t id);
/* Moves up to max finished results to out; waits up to wait_ms for one. */
int ev_server_poll(ev_server* s, ev_server_result* out, int32_t max, int32_t* count,
                   int32_t wait_ms);
int ev_server_resume(ev_server* s);
int ev_server_stats_get(ev_server* s, ev_server_stats* out);
/* Runs every admitted and pending request to completion, then frees. */
int ev_server_destroy(ev_server* s);

/* ---- measurement hooks (no reference counterpart) ------------------------
 * Used by benchmarks and profilers: events on the state's stream, the number
 * of kernels the engine has launched for a state, per-kernel-class timing
 * recorded with events around each launch while profiling is on, and pinned
 * host buffers for end-to-end copies. */
int ev_state_record_event(ev_state* s, int32_t slot); /* slot in [0, 16) */
int ev_state_elapsed_ms(ev_state* s, int32_t from_slot, int32_t to_slot, float* ms);
int ev_state_launch_count(const ev_state* s, uint64_t* out);

typedef struct ev_kernel_stat {
  char name[32];     /* kernel class, e.g. "tile_pass", "gate", "measure" */
  uint64_t launches; /* timed launches                                    */
  double ms;         /* summed event time                                 */
  double bytes;      /* summed algorithmic HBM bytes                      */
} ev_kernel_stat;
int ev_state_profile(ev_state* s, int32_t enable); /* enabling clears stats */
int ev_state_profile_read(ev_state* s, ev_kernel_stat* out, int32_t max, int32_t* count);

/* Measured FP64 FMA issue rate of the current device (FMA instructions per
 * second, from independent FMA chains on every SM): the roofline of the
 * complex128 kernels, whose arithmetic is FP64. */
int ev_probe_fp64(double* fma_per_s);
/* Checks the integer-pipe double product of the complex128 tile passes
 * against the FP64 pipe's on `count` operand pairs drawn from `seed`
 * (families that reach every rounding case); *mismatches = pairs whose bits
 * differ.  A check of the build, for tests. */
int ev_softfp_check(uint64_t seed, uint64_t count, uint64_t* mismatches);
/* The same check for the integer-pipe double add (softfp::add) against the
 * FP64 add, with second operands that cancel the first or sit at the
 * alignment's exponent gaps.  A check of the build, for tests. */
int ev_softfp_add_check(uint64_t seed, uint64_t count, uint64_t* mismatches);
/* Measured rate of the integer-pipe double add (adds per second, from
 * independent chains on every SM), beside ev_probe_fp64's FMA rate. */
int ev_probe_softadd(double* adds_per_s);
/* Checks the integer-pipe rounding of a double-float pair to f64 (the
 * complex64 sampling tree's leaves) against the FP64 add on `count` pairs;
 * *mismatches = pairs whose bits differ.  A check of the build, for tests. */
int ev_ff_check(uint64_t seed, uint64_t count, uint64_t* mismatches);
/* y = x W (rows x 64 times 64 x 64, row-major f64) in the digit-sliced
 * arithmetic of the EV_FUSED_OZAKI pass, restated on the host with the
 * kernel's own slicing and recombination routines.  A check of the build,
 * for tests; no reference counterpart. */
int ev_ozaki_gemm_host(const double* x, uint64_t rows, const double* w, double* y);
/* The same for the six-digit (digits = 6) or seven-digit (7) pass. */
int ev_ozaki_gemm_host_digits(const double* x, uint64_t rows, const double* w, double* y,
                              int32_t digits);
/* max_j |self_j - other_j| over two states of equal size, either amplitude
 * type (the max amplitude error of a complex64 run against complex128). */
int ev_max_abs_diff(const ev_state* self, const ev_state* other, double* out);

int ev_host_alloc(uint64_t bytes, void** out); /* page-locked host memory */
int ev_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* EVERETT_CUDA_H */
