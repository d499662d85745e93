/*
 * ls1gb300.h -- C ABI of the GB300 short-range molecular-dynamics engine.
 *
 * One context owns all device buffers and one CUDA stream for one periodic
 * (or open) box.  The engine replaces, for that box, the reference's
 *   LinkedCells container (binning, periodic halo, SoA caches),
 *   VectorizedCellProcessor (site-site LJ-12-6 / charge / dipole /
 *   quadrupole forces with reaction field, molecule-centre cut-off),
 *   FullMolecule::calcFM, the Leapfrog integrator and the local Upot/virial
 *   and kinetic-energy sums.
 * Every entry point returns MD_OK (0) or an MD_ERR_* code; md_last_error()
 * gives the message.  Host pointers are borrowed for the duration of the call
 * only.  Calls on one context must not overlap (the reference calls its
 * container from the master thread only).  No C++ exception crosses the ABI.
 *
 * Reference interfaces replaced (paths relative to the ls1-mardyn tree):
 *   md_create / md_destroy      LinkedCells::LinkedCells, ~LinkedCells
 *                               (src/particleContainer/LinkedCells.cpp:38-110)
 *   md_set_components           Domain::initParameterStreams -> Comp2Param::initialize
 *                               (src/Domain.cpp:629-631, src/molecules/Comp2Param.cpp:11-202)
 *                               and the VectorizedCellProcessor constructor's tables
 *                               (src/particleContainer/adapter/VectorizedCellProcessor.cpp:19-96)
 *   md_upload_molecules         ParticleContainer::addParticles (ParticleContainer.h:134)
 *   md_download_molecules       ParticleContainer::iterator (ParticleContainer.h:160)
 *   md_rebin_and_halo           LinkedCells::update (LinkedCells.cpp:241-355) +
 *                               DomainDecompBase::exchangeMolecules (DomainDecompBase.cpp:80-114) +
 *                               LinkedCells::updateMoleculeCaches (LinkedCells.cpp:1097-1107)
 *   md_get_cell_assignment      LinkedCells::getCellIndexOfMolecule/getCellIndexOfPoint
 *                               (LinkedCells.cpp:870-923)
 *   md_compute_forces           LinkedCells::traverseCells(VectorizedCellProcessor)
 *                               (LinkedCells.cpp:565-575) + Simulation::updateForces
 *                               (Simulation.cpp:835-845) + VCP::endTraversal (VCP.cpp:122-155)
 *   md_integrate_pre            Leapfrog::eventNewTimestep (Leapfrog.cpp:38-61)
 *   md_integrate_post           Leapfrog::eventForcesCalculated (Leapfrog.cpp:32-36, 63-147)
 *   md_run                      the hot part of Simulation::simulateOneTimestep
 *                               (Simulation.cpp:1076-1300) for an NVE run
 *   md_write_phasespace_binary  Domain::writeCheckpoint with the binary format
 *                               (src/Domain.cpp:581-625, FullMolecule::writeBinary
 *                               src/molecules/FullMolecule.cpp:448-470), as the
 *                               CheckpointWriter's `binary` type calls it
 *                               (src/io/CheckpointWriter.cpp:56-80)
 *   md_read_phasespace_binary   BinaryReader::readPhaseSpaceHeader + readPhaseSpace
 *                               (src/io/BinaryReader.cpp:76-343)
 *   md_planar_init/apply        Planar::init / calculateLongRange
 *                               (src/longRange/Planar.cpp:38-157, 223-460)
 */
#ifndef LS1GB300_H
#define LS1GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MD_OK 0
#define MD_ERR_ARG 1          /* invalid argument                                      */
#define MD_ERR_CUDA 2         /* CUDA runtime error                                    */
#define MD_ERR_CAPACITY 3     /* a capacity was exceeded; the context re-sizes on retry */
#define MD_ERR_STATE 4        /* calls out of order (e.g. forces before molecules)     */
#define MD_ERR_DEVICE 5       /* device status word: NaN, lost molecule, wait limit    */
#define MD_ERR_UNSUPPORTED 6  /* configuration the engine does not provide             */

#define MD_PREC_FP64 0        /* FP64 pair arithmetic and accumulation                 */
#define MD_PREC_MIXED 1       /* FP32 pair arithmetic, compensated per-molecule sums,
                                 FP64 positions, integration and global sums           */

#define MD_NUM_KINDS 7        /* LJ, C-C, C-D, D-D, C-Q, D-Q, Q-Q (FlopCounter order)  */

typedef struct md_ctx md_ctx;

typedef struct {
    double box_min[3];
    double box_max[3];
    double rc;          /* cutoffRadius: molecule-centre cut-off of the electrostatics and
                           lower bound of the cell edge                                   */
    double rc_lj;       /* LJ cut-off (molecule centres), <= rc                           */
    double eps_rf;      /* reaction-field permittivity epsilon_RF                         */
    int32_t periodic[3];/* 1: serial periodic halo in this dimension; 0: no halo (open)   */
    int32_t precision;  /* MD_PREC_FP64 or MD_PREC_MIXED                                  */
    int64_t capacity;   /* molecules to reserve (0: size from the first upload)           */
    double skin;        /* Verlet skin of the pair-candidate list; 0 rebuilds every step  */
    int32_t device;     /* CUDA device ordinal                                            */
    int32_t pair_scheme;/* MD_PAIRS_ROWS (0): per-molecule candidate rows, each pair
                           evaluated from both sides; MD_PAIRS_NEWTON3 (1): every pair
                           evaluated once (Newton's third law, as
                           VectorizedCellProcessor::processCellPair, VCP.cpp:2744-2819),
                           mixed precision only, with at least three list cells per periodic
                           dimension: by cluster pairs for one component of single-centre
                           LJ molecules with rc_lj = rc; by the higher-slot half of each
                           row, the neighbour's force, torque and virial added by FP32
                           atomics, for multi-site molecules; rows elsewhere.  The
                           atomics' order varies, so results agree between runs to FP32
                           rounding rather than bit for bit                                 */
} md_config;

#define MD_PAIRS_ROWS 0
#define MD_PAIRS_NEWTON3 1

/* One component (molecule type).  Site tables are row-major doubles:
 *   lj:         n_lj x 7         x y z m eps sigma shift6
 *   charge:     n_charge x 5     x y z m q
 *   dipole:     n_dipole x 7     x y z ex ey ez |mu|
 *   quadrupole: n_quadrupole x 7 x y z ex ey ez |Q|
 * Offsets are body-frame; orientation vectors are used as given (the
 * reference's ASCII reader does not normalise them).  inertia[d] > 0 overrides
 * the principal moment computed from the massive sites. */
typedef struct {
    int32_t n_lj, n_charge, n_dipole, n_quadrupole;
    const double* lj;
    const double* charge;
    const double* dipole;
    const double* quadrupole;
    double inertia[3];
} md_component;

typedef struct {
    int64_t n_inner;        /* molecules in the box                                      */
    int64_t n_halo;         /* periodic halo copies built                                */
    int64_t max_occupancy;  /* largest number of molecules in one cell                   */
    int64_t n_wrapped;      /* molecules moved back into the box this call               */
    int32_t cells[3];       /* cells per dimension including the halo layer              */
    int32_t reserved;
    double cell_length[3];
} md_bin_stats;

typedef struct {
    double upot;            /* Domain local Upot  = upot6lj/6 + upot_xpoles + my_rf      */
    double virial;          /* Domain local virial = virial_pairs + 3 my_rf              */
    double my_rf;           /* reaction-field term (-sum rffac e1.e2)                     */
    double upot6lj;
    double upot_xpoles;
    double virial_pairs;
    int64_t mol_pairs;      /* unique molecule pairs with centre distance^2 < rc^2       */
    int64_t site_pairs[MD_NUM_KINDS]; /* unique interacting site pairs per kind          */
} md_forces_out;

typedef struct {
    double summv2;          /* sum m v^2 over inner molecules                             */
    double sumIw2;          /* sum I w^2                                                 */
    int64_t n;
    int64_t rot_dof;
} md_kinetic_out;

typedef struct {
    double upot, virial, summv2, sumIw2;
} md_step_record;

int md_create(md_ctx** ctx, const md_config* cfg);
int md_destroy(md_ctx* ctx);
const char* md_last_error(const md_ctx* ctx);

/* mixing: ncomp*(ncomp-1)/2 rows of (xi, eta) for the pairs (i<j) in row order. */
int md_set_components(md_ctx* ctx, const md_component* comps, int32_t ncomp, const double* mixing);

/* Forces, torques and per-molecule virials (n x 3 each, in the order of the
 * last upload; NULL leaves a quantity unchanged), for a caller that uploaded
 * molecules between the force evaluation and the next pre-force half step --
 * ls1's host molecules after a plugin edited them through the container's
 * iterator -- since the pre-force half step kicks with the forces of the
 * last evaluation (FullMolecule::upd_preF, FullMolecule.cpp:331-361) and an
 * upload clears them. */
int md_set_forces(md_ctx* ctx, int64_t n, const double* F, const double* M, const double* Vi);

/* r, v, L: n x 3; q: n x 4 (w, x, y, z); comp: 0-based component index. */
int md_upload_molecules(md_ctx* ctx, int64_t n, const uint64_t* id, const int32_t* comp,
                        const double* r, const double* v, const double* q, const double* L);

/* Outputs in upload order; any pointer may be NULL.  F, M, Vi are those of the
 * last force evaluation. */
int md_download_molecules(md_ctx* ctx, int64_t n, uint64_t* id, int32_t* comp, double* r, double* v,
                          double* q, double* L, double* F, double* M, double* Vi);

/* ls1's binary phase-space (checkpoint) files, packed and unpacked on the
 * device.  Write: <prefix>.header.xml (time, box, molecule count, format
 * ICRVQD) and <prefix>.dat, one 116-byte record per molecule in upload order
 * (id u64, component u32 1-based, r[3] wrapped into the box, v[3], q[4]
 * w,x,y,z, L[3], little-endian doubles).  Read: a header/data pair in the
 * formats ICRVQD, ICRV or IRV replaces the context's molecules (components
 * must be set; the header's box must equal the context's to 1e-14 relative);
 * returns the header's time and the molecule count. */
int md_write_phasespace_binary(md_ctx* ctx, const char* prefix, double time);
int md_read_phasespace_binary(md_ctx* ctx, const char* header_path, const char* data_path, double* time,
                              int64_t* n);

/* Planar long-range correction for planar interfaces normal to y
 * (longRange/Planar.cpp, `<longrange type="planar">`).  md_planar_apply is
 * called after each md_compute_forces, where the reference calls
 * Planar::calculateLongRange (before calcFM): every `frequency` calls (the
 * first included) it samples the density profiles of the LJ centres and
 * dipolar components over `slabs` slabs and recomputes the slab corrections;
 * every call it adds each LJ centre's slab force to the y force (and its
 * torque) of molecules with y in [region_lo, region_hi], the slab virial to
 * every molecule's virial, and returns UpotCorr and VirialCorr (the values
 * the reference hands to Domain::setUpotCorr / setVirialCorr). */
typedef struct {
    int32_t slabs;             /* <slabs>                                                */
    int32_t frequency;         /* <frequency>: profile and corrections every n-th call   */
    double region_lo;          /* <region><left>: force corrections for y >= region_lo   */
    double region_hi;          /* <region><right>: ... and y <= region_hi (box: L_y)     */
    double target_temperature; /* thermostat-0 target temperature (dipole corrections)   */
} md_planar_config;
int md_planar_init(md_ctx* ctx, const md_planar_config* cfg);
int md_planar_apply(md_ctx* ctx, double* upot_corr, double* virial_corr);

int md_rebin_and_halo(md_ctx* ctx, md_bin_stats* stats);
int md_get_cell_assignment(md_ctx* ctx, int64_t n, int64_t* cell);
int md_compute_forces(md_ctx* ctx, md_forces_out* out);
int md_integrate_pre(md_ctx* ctx, double dt);
int md_integrate_post(md_ctx* ctx, double dt, md_kinetic_out* out);

/* nsteps full NVE steps on the device (pre-force half step, rebin + halo,
 * forces, post-force half step, sums) with no host synchronisation between
 * steps; rec (nsteps entries, may be NULL) receives the per-step sums. */
int md_run(md_ctx* ctx, double dt, int32_t nsteps, md_step_record* rec);

/* Adjoint of the force field at the current state (after md_compute_forces).
 * No counterpart in the reference, which has no gradients.  With upstream
 * gradients gU = dL/dUpot and gW = dL/dvirial (Upot and virial as reported by
 * md_compute_forces) and optionally gF (n x 3, dL/dF per molecule in upload
 * order, or NULL), it returns
 *   grad_r (n x 3, upload order, may be NULL):
 *       gU dUpot/dr + gW dvirial/dr + pair Hessian-vector products with gF
 *       (positions only; orientations held fixed),
 *   grad_params (nparam, may be NULL): gU dUpot/dp + gW dvirial/dp for the
 *       site parameters in the order: components in order, sites in the order
 *       LJ, charge, dipole, quadrupole; an LJ centre contributes (eps, sigma),
 *       a charge q, a dipole |mu|, a quadrupole |Q|.
 * nparam must equal that count (sum over components of 2 n_lj + n_charge +
 * n_dipole + n_quadrupole, at most 128).  Pairs are recomputed from the
 * pair-candidate list; nothing of the forward pass is stored. */
int md_adjoint(md_ctx* ctx, double gU, double gW, const double* gF, double* grad_r, double* grad_params,
               int32_t nparam);

/* ---- allocation-free force evaluation (no counterpart in the reference)
 * For callers that cannot allocate device memory: code recording into a CUDA
 * graph owned by a larger application, programs whose device memory comes
 * from their own pool, real-time drivers that forbid allocation after
 * start-up.  Computes, for a periodic box [0, box) of single-centre LJ
 * molecules (one component, centre at the molecule origin), the FP64 forces
 * d_F (n x 3, device), and d_upot_virial[0] = Upot, [1] = virial (device), as
 * md_compute_forces does, from device positions d_r (n x 3), on `stream`
 * (NULL: the default stream).  It allocates nothing: its scratch is one
 * file-scope device array of MD_NOALLOC_SCRATCH_BYTES that every GPU loading
 * the library keeps until exit.  Limits: n <= MD_NOALLOC_MAX_N, at least
 * three cells of edge >= rc per axis and at most MD_NOALLOC_MAX_CELLS cells;
 * larger problems return MD_ERR_CAPACITY, too few cells MD_ERR_UNSUPPORTED.
 * The first call on a device (with that device current) looks up the scratch
 * address and should come before any stream capture; so should the first
 * call after the device was reset or its context replaced, which looks the
 * address up again (the cache is keyed by the context's id).  All calls share the
 * scratch, which keeps the previous call's contents: calls that overlap on
 * the GPU race and must be serialised by the caller. */
#define MD_NOALLOC_MAX_N 131072
#define MD_NOALLOC_MAX_CELLS 65536
#define MD_NOALLOC_SCRATCH_BYTES 1966080
int md_forces_lj_noalloc(const double* d_r, int64_t n, const double box[3], double rc, double eps, double sigma,
                         double shift6, double* d_F, double* d_upot_virial, void* stream);

/* Homogeneous long-range correction (longRange/Homogeneous.cpp:22-146,
 * Homogeneous::init + calculateLongRange): UpotCorr and VirialCorr of the
 * current molecule counts, box volume, cut-offs and reaction field (what the
 * reference adds to the global Upot and virial in
 * Domain::calculateGlobalValues).  With add_to_molecule_virial != 0 it also
 * adds VirialCorr / (3 N) to every molecule's virial tensor diagonal, as the
 * reference does after each force evaluation.  MD_ERR_ARG when rc_lj does not
 * exceed the sum of two LJ centres' distances from their molecule centres. */
int md_longrange_homogeneous(md_ctx* ctx, int32_t add_to_molecule_virial, double* upot_corr, double* virial_corr);

/* Global velocity-scaling thermostat (the reference's VELSCALE_THERMOSTAT with
 * one thermostat: Domain::calculateGlobalValues, Domain.cpp:212-345, and
 * VelocityScalingThermostat::apply, VelocityScalingThermostat.cpp:67-96):
 * after the global sums of a step, beta_trans = (3 N T / sum m v^2)^0.4 and
 * beta_rot = (rotDOF T / sum I w^2)^0.4 scale v and the angular momenta, with
 * the reference's explosion heuristic when a beta falls below 0.9 (if
 * explosion_heuristics != 0).  md_set_thermostat: target <= 0 switches it off
 * (NVE) and resets the heuristic's counters; md_run then applies it every
 * step on the device.  md_apply_thermostat: one application after
 * md_integrate_post (the step-by-step path of the ls1 drop-in); returns the
 * betas. */
int md_set_thermostat(md_ctx* ctx, double target_temperature, int32_t explosion_heuristics);
int md_apply_thermostat(md_ctx* ctx, double* beta_trans, double* beta_rot);

/* Component-wise velocity-scaling thermostats (Domain::setComponentThermostat /
 * setTargetTemperature with ids >= 1, Domain::calculateGlobalValues and
 * VelocityScalingThermostat::apply with several thermostats): component c is
 * on thermostat component_thermostat[c] (1..nthermostats; every component
 * needs one), thermostat t has target target_temperatures[t - 1]; betas per
 * thermostat from its own sums, the explosion heuristic per thermostat with
 * counters shared as in the reference.  Replaces a global thermostat;
 * md_run and md_apply_thermostat then scale each molecule with its
 * thermostat's betas.  md_thermostat_betas reads the betas of the last
 * application (thermostat 0 = the global one). */
int md_set_thermostats(md_ctx* ctx, const int32_t* component_thermostat, int32_t nthermostats,
                       const double* target_temperatures, int32_t explosion_heuristics);
int md_thermostat_betas(md_ctx* ctx, int32_t thermostat, double* beta_trans, double* beta_rot);

/* Region-wise temperature control (thermostats/TemperatureControl: velocity
 * scaling per control region and slab).  A region is the open box lower <
 * r < upper; its molecules of `component` (1-based; 0 = all) are binned in
 * `numslabs` slabs along y.  Every `frequency`-th step with start < step <
 * stop (Init/MeasureKineticEnergy/CalcGlobalValues) the sums per slab give
 * beta_trans = (ndir N T / sum m v_d^2)^exponent over the thermostated
 * directions d (bits 1 = x, 2 = y, 4 = z) and beta_rot = (rotDOF T / sum I
 * w^2)^exponent (1 for an empty slab or no rotational DOF); for start < step
 * <= stop (ControlTemperature) those directions of v are scaled by 2 -
 * 1/beta_trans and L by 2 - 1/beta_rot, region by region
 * (TemperatureControl.cpp:241-427, 666-770).  T follows the region's ramp
 * (start -> end between update_start and update_stop, every update_freq
 * steps) when ramp_enabled.  Replaces the global and component-wise
 * thermostats inside md_run (Simulation.cpp:1236-1268), applied after each
 * step's global values; md_set_simstep sets the step number of the state
 * (md_run's steps are step + 1, step + 2, ...).  md_temperature_control_betas
 * reads the betas of region r's slabs of the last measurement.
 * A region with method MD_TC_ANDERSEN (ControlRegionT::ControlTemperature,
 * TemperatureControl.cpp:411-419) neither measures nor uses slabs,
 * directions, exponent or ramp: at each control step every molecule inside
 * it is selected with probability nu * timestep and gets v_d = g * sqrt(T/m)
 * and L_d = g' * sqrt(T/m) for d = x, y, z with independent standard normal
 * g, g' (the reference's shared reserve deviate gives L the translational
 * deviation too).  The reference draws from one sequential generator in
 * traversal order; here the draws of molecule `id` at step s in region r
 * are a counter-based stream keyed by (seed, s, id, r), so a run does not
 * depend on the order or the number of threads. */
#define MD_TC_MAX_REGIONS 8
#define MD_TC_MAX_SLABS 64
#define MD_TC_VELOCITY_SCALING 0
#define MD_TC_ANDERSEN 1
typedef struct {
    double lower[3], upper[3];
    double target_temperature;
    int32_t component;          /* 1-based component id, 0 = every component */
    int32_t numslabs;           /* 1 .. MD_TC_MAX_SLABS                        */
    double exponent;
    int32_t directions;         /* bit mask: 1 = x, 2 = y, 4 = z               */
    int32_t ramp_enabled;
    double ramp_start, ramp_end;
    int64_t ramp_update_start, ramp_update_stop, ramp_update_freq;
    int32_t method;             /* MD_TC_VELOCITY_SCALING or MD_TC_ANDERSEN    */
    int32_t reserved;
    double nu;                  /* Andersen collision frequency                */
} md_tc_region;
typedef struct {
    int64_t start, frequency, stop;
    int32_t nregions;
    int32_t reserved;
    md_tc_region regions[MD_TC_MAX_REGIONS];
    double timestep;            /* integrator time step (Andersen regions)     */
    uint64_t seed;              /* Andersen draws                              */
} md_temperature_control;
int md_set_temperature_control(md_ctx* ctx, const md_temperature_control* tc);
int md_set_simstep(md_ctx* ctx, int64_t simstep);
/* md_apply_temperature_control: the temperature control of step `simstep`
 * for callers that step with the half-step calls (after md_integrate_post,
 * as Simulation::simulateOneTimestep calls TemperatureControl). */
int md_apply_temperature_control(md_ctx* ctx, int64_t simstep);
int md_temperature_control_betas(md_ctx* ctx, int32_t region, double* beta_trans, double* beta_rot);

/* Wait for all work of the context. */
int md_sync(md_ctx* ctx);

/* ---- reduced memory mode (the reference's ENABLE_REDUCED_MEMORY_MODE build:
 * MoleculeRMM, VCP1CLJRMM, LeapfrogRMM).  One component with a single LJ
 * centre at the molecule centre (in mixed precision rc_lj = rc); forces are
 * never stored.
 * md_rmm_forces: VCP1CLJRMM traversal (VCP1CLJRMM.cpp:88-369): rebin and
 *   rebuild when due, pair kernel that adds dt_inv_m * F to every velocity.
 *   Simulation::prepare_start passes dt/(2m) for the initial force pass,
 *   LeapfrogRMM steps dt/m (Simulation.cpp:902-938, VCP1CLJRMM.cpp:41-44).
 *   Upot, virial and pair counts as md_compute_forces.  Replaces
 *   VCP1CLJRMM::processCellPair/processCell/endTraversal.
 * md_rmm_positions: r += dt v (LeapfrogRMM::computePositions,
 *   PositionCellProcessorRMM.h:33-60).
 * md_rmm_velocities: N and sum v.v, without the mass
 *   (LeapfrogRMM::computeVelocities, VelocityCellProcessorRMM.h:95-128);
 *   sumIw2 = 0, rot_dof = 0.
 * md_rmm_run: nsteps LeapfrogRMM steps (positions, rebin when due, forces
 *   with dt/m, velocity sums) as CUDA graphs; rec[k].summv2 = sum v.v. */
int md_rmm_forces(md_ctx* ctx, double dt_inv_m, md_forces_out* out);
int md_rmm_positions(md_ctx* ctx, double dt);
int md_rmm_velocities(md_ctx* ctx, md_kinetic_out* out);
int md_rmm_run(md_ctx* ctx, double dt, int32_t nsteps, md_step_record* rec);

/* ---- measurement hooks (no counterpart in the reference; used by bench.py)
 * md_get_stream: the CUDA stream (cudaStream_t) every kernel of the context
 * runs on, so a caller can bracket calls with its own CUDA events.
 * md_time_kernels: mean device time of each kernel family, measured with
 * CUDA events on that stream over `reps` back-to-back launches on the current
 * state (the pair-candidate list is left as it is). */
typedef struct {
    double force_ms;          /* one pair-kernel launch (k_force_*)                     */
    double pre_ms;            /* one pre-force Leapfrog half step                       */
    double post_ms;           /* one post-force half step + sums                        */
    double rebuild_ms;        /* one forced rebin + list rebuild                        */
    double mean_candidates;   /* mean pair-candidate list length per molecule           */
    int64_t rebuilds;         /* list rebuilds since md_create                          */
    int32_t launches_per_step;/* kernels one graph-captured md_run step launches when
                                 no list rebuild is due                                 */
    int32_t launches_per_rebuild; /* kernels a list rebuild adds to such a step         */
    double adjoint_ms;        /* one md_adjoint kernel pass (gU = gW = 1, no gF),
                                 without its host copies                                */
    double step_force_ms;     /* the pair evaluation of one md_run step of one component of
                                 single-centre LJ molecules in mixed precision with both
                                 Leapfrog half steps: the pair kernel with the half steps
                                 fused (rows), or the Newton-3 pair kernel plus its
                                 half-step kernel (cluster pairs); 0 otherwise          */
    double lf_ms;             /* cluster pairs: that half-step kernel alone; 0 otherwise */
    int32_t pair_scheme;      /* the scheme the context's pair evaluations use now:
                                 MD_PAIRS_NEWTON3 (cluster pairs, or half rows of
                                 multi-site molecules) or MD_PAIRS_ROWS                  */
    int32_t cluster_size;     /* molecules per cluster of the Newton-3 path             */
} md_kernel_times;

int md_get_stream(md_ctx* ctx, void** stream);
/* md_rebuilds: list rebuilds since md_create (device counter, read after the
 * stream's work so far). */
int md_rebuilds(md_ctx* ctx, int64_t* count);
int md_time_kernels(md_ctx* ctx, int32_t reps, md_kernel_times* out);

/* ---- batches of independent boxes (no counterpart in the reference, which
 * runs one domain per process).  Many periodic boxes of single-centre LJ
 * molecules (one component: eps, sigma, mass; rc_lj = rc) are advanced
 * together: every kernel launch covers all boxes, a run is captured as CUDA
 * graphs of `graph_steps` steps, and per-box Upot / virial / sum m v^2 are
 * recorded every step.  Each box follows the md_ctx semantics of the same
 * box run alone (LinkedCells + VectorizedCellProcessor::_loopBodyLJ,
 * VectorizedCellProcessor.cpp:171-224; Leapfrog, Leapfrog.cpp:38-147).
 *
 * md_batch_create: box b spans [0, box_len[3b+d]) along d, periodic; every box
 *   needs three list cells of edge (rc + skin) per axis (skin is lowered to fit;
 *   a box shorter than 3 rc is an error).  skin < 0 picks 0.3 (or the largest
 *   that fits); threads_per_molecule 0 picks 1.  On error *b is still set so
 *   md_batch_last_error can be read; call md_batch_destroy in every case.
 * md_batch_upload: molecules of box k are rows [box_start[k], box_start[k+1])
 *   of r, v (n x 3, n = box_start[nbox]); ids may be NULL (1..n).
 * md_batch_compute_forces: forces at the uploaded positions (the reference's
 *   Simulation::prepare_start); out[nbox] (may be NULL) gets Upot, virial and
 *   the number of interacting pairs of each box.
 * md_batch_run: nsteps NVE Leapfrog steps; rec (may be NULL) is nsteps x nbox,
 *   row-major by step.
 * md_batch_download: upload order; any pointer may be NULL.
 * md_batch_autotune: coordinate descent over the list skin (list cell edge
 *   rc + skin: 0.1 ... 0.5 as the boxes allow), the list-cell occupancy in
 *   dilute boxes (0, 8, 16, 32) and the threads per molecule row (1, 2, 4; 1
 *   only in FP64): `trial_steps` steps timed per candidate, the state restored
 *   after each trial, the fastest kept; out (may be NULL) lists every trial. */
typedef struct md_batch md_batch;

typedef struct {
    int32_t nbox;
    int32_t precision;            /* MD_PREC_FP64 or MD_PREC_MIXED */
    const double* box_len;        /* nbox x 3 */
    double rc;                    /* molecule-centre cut-off (also the LJ cut-off) */
    double epsilon, sigma, mass;  /* the LJ centre */
    int32_t shifted;              /* 1: LJ shifted to zero at rc (LJTS) */
    int32_t threads_per_molecule; /* 0, 1, 2 or 4 */
    double skin;                  /* pair-candidate list skin; < 0: default */
    int32_t device;
    int32_t reserved;
    double cell_occupancy;        /* > 0: dilute boxes get list cells of about this many molecules */
} md_batch_config;

typedef struct {
    double upot;
    double virial;
    int64_t pairs;
} md_box_sums;

#define MD_BATCH_TUNE_MAX 16
typedef struct {
    double skin;                  /* chosen */
    int32_t threads_per_molecule; /* chosen */
    int32_t ntrials;
    double ms_per_step;           /* of the chosen configuration */
    double trial_skin[MD_BATCH_TUNE_MAX];
    int32_t trial_tpm[MD_BATCH_TUNE_MAX];
    double trial_ms_per_step[MD_BATCH_TUNE_MAX];
    double cell_occupancy;        /* chosen */
    double trial_occupancy[MD_BATCH_TUNE_MAX];
} md_batch_tuning;

int md_batch_create(md_batch** b, const md_batch_config* cfg);
int md_batch_destroy(md_batch* b);
const char* md_batch_last_error(const md_batch* b);
int md_batch_upload(md_batch* b, const int64_t* box_start, const uint64_t* ids, const double* r, const double* v);
int md_batch_compute_forces(md_batch* b, md_box_sums* out);
int md_batch_run(md_batch* b, double dt, int32_t nsteps, int32_t graph_steps, md_step_record* rec);
int md_batch_download(md_batch* b, uint64_t* ids, double* r, double* v, double* F);
int md_batch_autotune(md_batch* b, double dt, int32_t trial_steps, md_batch_tuning* out);
int md_batch_get_stream(md_batch* b, void** stream);
int md_batch_rebuilds(md_batch* b, int64_t* count);

#ifdef __cplusplus
}
#endif

#endif /* LS1GB300_H */
