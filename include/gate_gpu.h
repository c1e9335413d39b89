/*
 * gate_gpu.h - C ABI of the GB300 photon-transport path (libgategpu.so).
 *
 * One context drives one CUDA device.  Every function returns a status code
 * (GG_OK on success); on failure gg_last_error() gives the message.  Callers
 * own every host buffer they pass in; nothing is retained past a call (the
 * context keeps device copies).  Calls on one context are not re-entrant.
 *
 * The functions replace the following reference interfaces (paths relative
 * to the opengate project):
 *   gg_create / gg_destroy      SimulationEngine.initialize / close
 *                               (opengate/engines.py:1721, 1414)
 *   gg_upload_tables            physics-table build inside G4RunManager::Initialize
 *                               for physics_list_name="G4EmStandardPhysics"
 *                               (opengate/physics.py:341-347); the per-material
 *                               cross sections Geant4 computes internally
 *   gg_upload_volume            ImageVolume.construct + create_label_image +
 *                               GateImageNestedParameterisation::ComputeMaterial
 *                               (opengate/geometry/volumes.py:1050, 1200-1243;
 *                               core/opengate_core/opengate_lib/GateImageNestedParameterisation.cpp:47-75)
 *   gg_set_world                world volume (opengate/managers.py:1435 VolumeManager)
 *   gg_set_source               GateGenericSource::InitializePosition/Direction/Energy
 *                               (core/opengate_core/opengate_lib/GateGenericSource.cpp:312-664)
 *   gg_set_source, position type GG_POS_VOXELS
 *                               GateVoxelSource / GateSPSVoxelsPosDistribution
 *                               (core/opengate_core/opengate_lib/GateSPSVoxelsPosDistribution.cpp:29-74)
 *   gg_add_dose_tally           GateDoseActor::InitializeCpp / BeginOfRunAction
 *                               (core/opengate_core/opengate_lib/GateDoseActor.cpp:100-137)
 *   gg_spect_set_free_flight    GateGammaFreeFlightOptrActor (biasing/GateGammaFreeFlightOptn.cpp:34-83)
 *   gg_spect_set_blur           GateDigitizerBlurringActor / GateDigitizerSpatialBlurringActor
 *                               (core/opengate_core/opengate_lib/digitizer/*BlurringActor.cpp)
 *   gg_set_tle                  GateTLEDoseActor (track-length estimator)
 *                               (core/opengate_core/opengate_lib/GateTLEDoseActor.cpp:174-299)
 *   gg_run                      GateSourceManager::StartMasterThread -> /run/beamOn
 *                               (core/opengate_core/opengate_lib/GateSourceManager.cpp:198-244)
 *                               with GateDoseActor::SteppingAction / ScoreSquaredValue /
 *                               FlushSquaredValues (GateDoseActor.cpp:180-243, 359-397)
 *   gg_get_image                DoseActor.EndOfRunActionMasterThread -> fetch_from_cpp_image
 *                               (opengate/actors/doseactors.py:662-715)
 *   gg_get_counters             SimulationStatisticsActor counts
 *                               (core/opengate_core/opengate_lib/GateSimulationStatisticsActor.cpp:53-201)
 */
#ifndef GATE_GPU_H
#define GATE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GG_OK 0
#define GG_ERR_ARG 1
#define GG_ERR_CUDA 2
#define GG_ERR_QUEUE_OVERFLOW 3
#define GG_ERR_TIMEOUT 4
#define GG_ERR_DOMAIN 5
#define GG_ERR_STATE 6

/* precision of a context's transport arithmetic */
#define GG_PREC_F32 32
#define GG_PREC_F64 64

/* source position types (GenericSource position.type) */
#define GG_POS_POINT 0
#define GG_POS_BOX 1
#define GG_POS_SPHERE 2
#define GG_POS_DISC 3
#define GG_POS_VOXELS 4 /* VoxelSource: activity image, 3-level CDF */

/* direction types (GenericSource direction.type) */
#define GG_DIR_ISO 0
#define GG_DIR_MOMENTUM 1
#define GG_DIR_FOCUSED 2
/* ForceDirection policy of the angular acceptance toward the SPECT heads
   (GateForcedDirectionManager.cpp, contrib/spect/spect_config.py:986-1006
   setup_force_direction: one source copy per head): the photon of history h
   is aimed at head h mod n_heads, cos(theta) uniform in [fd_cos_max,
   fd_cos_min] about the head's axis at the history's run, phi uniform, and
   starts with weight (fd_cos_min - fd_cos_max) / 2.  With primary free
   flight only (the weight needs the weighted tallies). */
#define GG_DIR_FORCED 3

/* energy types (GenericSource energy.type) */
#define GG_ENE_MONO 0
#define GG_ENE_LINES 1     /* "spectrum_discrete" */
#define GG_ENE_HISTOGRAM 2 /* "spectrum_histogram", no interpolation */
#define GG_ENE_RANGE 3

/* images returned by gg_get_image */
#define GG_IMG_EDEP 0
#define GG_IMG_EDEP_SQUARED 1
#define GG_IMG_DOSE 2          /* dose grid with score_dose: sum of edep / rho (MeV cm3 / g) */
#define GG_IMG_DOSE_SQUARED 3  /* its history-by-history squares */

/* counters returned by gg_get_counters (uint64 slots) */
#define GG_CNT_HISTORIES 0
#define GG_CNT_WOODCOCK_STEPS 1 /* tentative collision points inside the image */
#define GG_CNT_REAL_INTERACTIONS 2
#define GG_CNT_DEPOSITS 3       /* energy deposits (> 0) inside the image */
#define GG_CNT_TALLY_ENTRIES 4  /* per-history voxel entries flushed to the tally */
#define GG_CNT_LIST_OVERFLOWS 5 /* per-history list flushed before the history ended */
#define GG_CNT_WORLD_STEPS 6
#define GG_CNT_ESCAPED 7
#define GG_CNT_SKIPPED 8        /* directions rejected by angular acceptance */
#define GG_CNT_LOOP_CAPPED 9    /* sampling loops stopped at their iteration cap */
#define GG_CNT_STACK_OVERFLOW 10
#define GG_CNT_SECONDARIES 11   /* annihilation photons created */
#define GG_CNT_HEAD_STEPS 12    /* transport steps inside SPECT heads */
#define GG_CNT_SINGLES 13       /* events with energy deposited in a crystal */
#define GG_CNT_ARF_PHOTONS 14   /* photons at a collimator face scored by the ARF network */
#define GG_CNT_ARF_FALLBACK 15  /* photons at a head the ARF stage left to plain tracking */
#define GG_N_COUNTERS 16

/* Physics tables: see opengate_gb300/tables.py for the contract. */
typedef struct {
  int32_t n_e;          /* energy grid points */
  float ln_emin;        /* ln(E_min / MeV) */
  float inv_dln;        /* (n_e - 1) / ln(E_max / E_min) */
  float e_min;          /* MeV, photons below are absorbed locally */
  float e_max;          /* MeV */
  int32_t n_comp;
  const float *sig;      /* [n_comp][n_e] mm^-1 per g/cm3 */
  const float *cum;      /* [n_comp][3][n_e] Compton, +photo, +Rayleigh */
  const float *ray_amax; /* [n_comp][n_e] Rayleigh cumulative reached at E (x^2 = (E/hc)^2) */
  int32_t n_ray;         /* Rayleigh x^2 grid points */
  const float *ray_x2;   /* [n_ray] increasing x^2 nodes in 1/Angstrom^2, ray_x2[0] = 0 */
  const float *ray_cum; /* [n_comp][n_ray] normalised cumulative of F^2 dx^2 at the nodes */
  int32_t n_mat;
  const int32_t *mat_comp; /* [n_mat] */
  const float *mat_rho;    /* [n_mat] g/cm3 */
} gg_tables_desc;

/* Voxelised image volume, axis aligned, labels index the material table. */
typedef struct {
  int32_t dims[3];          /* nx, ny, nz (x fastest in memory) */
  double spacing[3];        /* mm */
  double corner[3];         /* mm, world position of the outer corner of voxel (0,0,0) */
  const uint16_t *labels;   /* [nz][ny][nx] material index per voxel */
  const float *majorant;    /* [n_e] mm^-1, >= every label's attenuation */
} gg_volume_desc;

/* World box (centred at the origin) and its material. */
typedef struct {
  double half_size[3]; /* mm */
  int32_t material;    /* index into the material table */
} gg_world_desc;

typedef struct {
  /* position */
  int32_t pos_type;
  double translation[3]; /* mm */
  double rotation[9];    /* row-major, local -> world */
  double half_size[3];   /* box half sizes, mm */
  double radius;         /* sphere / disc, mm */
  /* direction */
  int32_t dir_type;
  double theta[2]; /* rad, iso */
  double phi[2];   /* rad, iso */
  double momentum[3];
  double focus[3];
  /* angular acceptance ("Rejection" policy, "SkipEvents"): the direction is
     re-sampled until the ray from the vertex crosses one of the boxes */
  int32_t n_accept;
  const double *accept_boxes; /* [n_accept][6]: min xyz, max xyz (world, mm) */
  int32_t max_rejection;
  /* energy */
  int32_t ene_type;
  double mono;          /* MeV */
  int32_t n_spec;       /* lines: n energies; histogram: n bins */
  const double *spec_e; /* lines: [n]; histogram: [n+1] edges; MeV */
  const double *spec_cdf; /* [n], normalised cumulative weights */
  double e_lo, e_hi;    /* range */
  /* GG_POS_VOXELS (GateSPSVoxelsPosDistribution): voxel (k, j, i) chosen by
     lower_bound on cdf_z, then cdf_y[i], then cdf_x[i][j] (draws in (0, 1]),
     position = corner + (index + 0.5) * spacing + (u - 0.5) * spacing */
  int32_t vox_dims[3];      /* nx, ny, nz of the activity image */
  double vox_spacing[3];    /* mm */
  double vox_corner[3];     /* mm, outer corner of voxel (0, 0, 0), world */
  const float *cdf_z;       /* [nz] */
  const float *cdf_y;       /* [nz][ny] */
  const float *cdf_x;       /* [nz][ny][nx] */
  /* GG_DIR_FORCED: cosines of angle_tolerance_min and angle_tolerance_max */
  double fd_cos_min, fd_cos_max;
} gg_source_desc;

/* SPECT heads: parallel-hole collimator + crystal, and the projection digitizer
   (Hits -> Adder EnergyWinnerPosition -> EnergyWindows -> Projection).
   Head-local frame: w along the head's outward normal with the collimator
   front face at w = 0, (a1, a2) along the detector axes e1, e2.  The head box
   is |a1|, |a2| <= half_width, 0 <= w <= collimator + gap + crystal.  The
   collimator is the collimator material with hexagonal holes (vacuum) of
   apothem hole_apothem on two rectangular lattices of pitch (pitch_x,
   pitch_y), the second shifted by half a pitch in both axes; hole faces are
   normal to 30, 90 and 150 degrees in the (a1, a2) plane. */
typedef struct {
  double half_width;           /* mm */
  double collimator_thickness; /* mm */
  double gap;                  /* mm, vacuum between collimator and crystal */
  double crystal_thickness;    /* mm */
  double hole_apothem;         /* mm (flat-to-flat / 2) */
  double pitch_x, pitch_y;     /* mm */
  int32_t collimator_material; /* material table index */
  int32_t crystal_material;    /* material table index */
  int32_t n_windows;           /* <= 8 */
  double window_lo[8];         /* MeV, window k = [lo, hi) */
  double window_hi[8];
  int32_t size[2];             /* projection pixels along e1, e2 */
  double spacing[2];           /* mm */
  int32_t n_heads;             /* 1 or 2 */
  int32_t n_runs;              /* gantry positions; projection slice = window + run * n_windows */
  int32_t adder_policy;        /* GG_ADDER_WINNER (0) or GG_ADDER_CENTROID: position of a single */
  /* Head housing (replaces the shielding box of add_spect_box,
     contrib/spect/ge_discovery_nm670.py:215-262): slabs across the head's
     width, an entrance cover between the gap and the crystal and up to four
     layers behind the crystal (reflector, back compartment, lead cover and
     steel shielding backs), outwards from the crystal; interactions there
     are tracked like the collimator's, deposits outside the crystal are not
     scored.  No layers (all zero): collimator, gap and crystal only. */
  int32_t n_cover;             /* 0 or 1 */
  double cover_thickness;      /* mm */
  int32_t cover_material;      /* material table index */
  int32_t n_back;              /* 0..4 */
  double back_thickness[4];    /* mm, from the crystal outwards */
  int32_t back_material[4];
  /* 1: the side faces of the head box absorb (the shielding box's lead and
     steel rims around the crystal, 3-18 mm of lead plus 20 mm of steel:
     below 1 % transmission at 208 keV, taken as black walls): a photon that
     would enter or leave a head through a side face stops there.  0: the
     sides are open (photons enter the crystal from the side). */
  int32_t shielded_sides;
} gg_spect_desc;
/* adder policies (GateDigiAdderInVolume, digitizer/GateDigiAdderInVolume.cpp:29-88) */
#define GG_ADDER_WINNER 0   /* EnergyWinnerPosition: the largest deposit's point */
#define GG_ADDER_CENTROID 1 /* EnergyWeightedCentroidPosition: sum(e x) / sum(e) */

/* ARF training photons (replaces the source + plane of
   contrib/spect/ge_discovery_nm670.py:994-1027 add_source_for_arf_training_dataset /
   add_actor_for_arf_training_dataset): photons start on the collimator front
   face of one head, position uniform in |a1| <= half_extent[0],
   |a2| <= half_extent[1], direction in the cone theta <= acos(cos_theta_max)
   about the head normal (into the head) - isotropic, or with theta uniform
   in [0, theta_max] when theta_uniform is set (more rows near the hole axis,
   where the detection probability varies; the network learns the window
   probability given the direction, which does not depend on how the
   directions were drawn) - and energy uniform in [e_min, e_max]. */
typedef struct {
  double e_min, e_max;      /* MeV */
  double cos_theta_max;
  double half_extent[2];    /* mm */
  double russian_roulette;  /* rows of photons detected in no window are kept with probability 1 / this (>= 1) */
  int32_t theta_uniform;    /* 0: isotropic directions, 1: theta uniform */
} gg_arf_sampling;

typedef struct gg_ctx gg_ctx;

typedef struct {
  int32_t device;     /* CUDA device ordinal */
  int32_t precision;  /* GG_PREC_F32 or GG_PREC_F64 */
  int32_t block_size; /* 0 = default */
  int32_t blocks_per_sm; /* 0 = default */
  int32_t chunk;      /* histories a warp claims per queue fetch, 0 = default */
  int64_t batch;      /* histories per tally batch, 0 = default (2^26; buffers sized to min(batch, run)) */
  int32_t refill_min;   /* 1..32: lanes waiting for a history that trigger a refill phase, 0 = default */
  int32_t interact_min; /* 1..32: pending collisions that trigger an interaction phase, 0 = default */
} gg_device_opts;

/* Dose transport kernel of gg_run for single simulations with analog scoring
   (the track-length estimator and batched simulations always use the phase
   kernel).  Both give identical results; they differ in speed only. */
#define GG_KERNEL_WAVEFRONT 0 /* per-block wavefront compacted by event type */
#define GG_KERNEL_PHASED 1    /* block-synchronous phases, one history per thread (default) */

int gg_create(const gg_device_opts *opts, gg_ctx **out);
int gg_destroy(gg_ctx *ctx);
/* Copies the last error message of ctx (or of the last failed gg_create if
   ctx is NULL) into buf, always NUL-terminated. */
int gg_last_error(const gg_ctx *ctx, char *buf, size_t len);

/* The tables stay in each transport block's shared memory beside its two
   per-history voxel lists: sizeof(real) * (n_comp * n_e + n_e + n_mat) +
   4 * n_mat bytes (16-byte aligned) plus 2 * 8 * 256 * (4 + sizeof(real))
   must not exceed 200 KiB (GG_ERR_ARG otherwise). */
int gg_upload_tables(gg_ctx *ctx, const gg_tables_desc *tables);
int gg_upload_volume(gg_ctx *ctx, const gg_volume_desc *volume);
int gg_set_world(gg_ctx *ctx, const gg_world_desc *world);
int gg_set_source(gg_ctx *ctx, const gg_source_desc *source);
/* Enables the edep / edep-squared tally on the image grid and zeroes it. */
int gg_add_dose_tally(gg_ctx *ctx, int32_t score_squared);
/* Dose tally on a grid of its own (replaces the DoseActor placement of
   GateDoseActor::BeginOfRunActionMasterThread + AttachImageToVolume and
   GetVoxelPosition, core/opengate_core/opengate_lib/GateDoseActor.cpp:88-178,
   GateHelpersImage.txx:20-58): dims voxels of `spacing`, outer corner
   `corner` (world, mm), axis-aligned with the image.  A deposit in the
   image is scored in the grid voxel of the interaction point, or not at all
   outside the grid; score_dose adds the dose tally sum(edep / rho) of the
   material at the point (GG_IMG_DOSE, GG_IMG_DOSE_SQUARED).  gg_get_image then
   returns grid-sized images.  NULL or dims[0] = 0: back to the image grid.
   Not with the track-length estimator or batched simulations. */
typedef struct {
  int32_t dims[3];
  double spacing[3]; /* mm */
  double corner[3];  /* mm, world position of the outer corner of voxel (0, 0, 0) */
  int32_t score_dose;
} gg_dose_grid_desc;
int gg_set_dose_grid(gg_ctx *ctx, const gg_dose_grid_desc *grid);

/* Selects the dose transport kernel (GG_KERNEL_*); no counterpart in the
   reference (Geant4 has one stepping loop). */
int gg_set_transport_kernel(gg_ctx *ctx, int32_t kind);
int gg_reset_tally(gg_ctx *ctx);

/* Track-length estimator of the dose tally (replaces the TLEDoseActor:
   GateTLEDoseActor::SteppingAction / ScoreTLEDepositStep,
   core/opengate_core/opengate_lib/GateTLEDoseActor.cpp:174-299, options of
   opengate/actors/doseactors.py:722-776).  With enabled = 1 a photon inside
   the image whose energy is at or below threshold_energy scores
   E * mu_en(E, material) * length in every voxel its paths cross, and the
   energy it gives to electrons at its interactions is not scored; photons
   above the threshold score as without the estimator.  A scored photon at or
   below energy_min deposits its energy in its voxel and stops.  mu_en comes
   from `muen` ([n_comp][n_e], mm^-1 per g/cm3, the grid and compositions of
   the uploaded tables).  Single (not batched) dose runs only; enabled = 0
   switches it off. */
typedef struct {
  int32_t enabled;
  double threshold_energy; /* MeV; +inf scores every photon (threshold type "None") */
  double energy_min;       /* MeV */
  const float *muen;       /* [n_comp][n_e] */
} gg_tle_desc;
int gg_set_tle(gg_ctx *ctx, const gg_tle_desc *tle);
/* Simulates histories [first_history, first_history + n) with the given seed
   and adds them to the tally.  Histories are processed in batches (the
   context's batch size); the result does not depend on launch parameters. */
int gg_run(gg_ctx *ctx, uint64_t n_histories, uint64_t seed, uint64_t first_history);
int gg_synchronize(gg_ctx *ctx);
int gg_get_image(gg_ctx *ctx, int32_t which, double *out, size_t n);
/* The device copy of an image (GG_IMG_*): *ptr = its FP64 voxels on the
   context's device, *n = their number; the context's stream is synchronised
   first.  The pointer stays valid until the next gg_run, gg_reset_tally,
   tally change or gg_destroy.  For merging replicas on the device (an
   all-reduce over the ranks' images, opengate/engines.py's merge of the
   processes' actor outputs) without a round trip through the host. */
int gg_get_image_device(gg_ctx *ctx, int32_t which, void **ptr, size_t *n);
int gg_get_counters(gg_ctx *ctx, uint64_t *out, size_t n);
/* Page-locked host memory (cudaMallocHost) for callers that download or
   upload the same buffers repeatedly: copies from and to it run at the host
   link's DMA rate instead of through the driver's staging of pageable
   memory.  gg_host_alloc returns NULL on failure; gg_host_free(NULL) is a
   no-op.  No reference counterpart (the reference's images live in host
   memory). */
void *gg_host_alloc(size_t bytes);
int gg_host_free(void *ptr);
/* Device time (CUDA events on the context's stream) of the last gg_run, ms:
   source stage, transport kernel and tally flush, summed over batches, and
   the number of kernel launches. */
int gg_last_kernel_ms(gg_ctx *ctx, double *generate_ms, double *transport_ms, double *flush_ms,
                      int32_t *launches);

/* SPECT (replaces the NM670 head of contrib/spect/ge_discovery_nm670.py:125-164,
   464-490 and GateDigitizerHitsCollectionActor / GateDigiAdderInVolume /
   GateDigitizerEnergyWindowsActor / GateDigitizerProjectionActor,
   core/opengate_core/opengate_lib/digitizer/*.cpp).  gg_spect_setup enables
   the head transport and zeroes the projection counts and the counters; the
   dose tally is not needed.  gg_spect_set_heads places the heads for one run (gantry position):
   frames[n_heads][12] = collimator front-face centre xyz, outward normal xyz,
   e1 xyz, e2 xyz (world, unit vectors); the following gg_run calls score into
   that run's slices.  gg_spect_run simulates every run in one call (the
   reference's run_timing_intervals loop with one head position per run,
   contrib/spect/ge_discovery_nm670.py:1056-1080 rotate_gantry): run r gets
   histories [first + r n_per_run, first + (r + 1) n_per_run) and the head
   frames frames[r][n_heads][12] (NULL: the frames given so far by
   gg_spect_set_heads); all runs go through one set of launches, so results
   equal n_runs gg_spect_set_heads + gg_run calls with the same histories.
   gg_get_projection returns the counts as float64,
   [head][run][window][size[1]][size[0]]. */
int gg_spect_setup(gg_ctx *ctx, const gg_spect_desc *spect);

/* Digitizer blurring of the singles, between the adder and the energy
   windows (replaces DigitizerBlurringActor on TotalEnergyDeposit and
   DigitizerSpatialBlurringActor on PostPosition:
   digitizer/GateDigitizerBlurringActor.cpp:74-97,
   digitizer/GateDigitizerSpatialBlurringActor.cpp:85-206,
   opengate/actors/digitizers.py:428-580, 801-920).  Energy: E' = N(E, sigma)
   with sigma = energy_sigma (GG_BLUR_GAUSSIAN), or FWHM/E =
   resolution sqrt(reference) / sqrt(E) (GG_BLUR_INVERSE_SQUARE), or
   slope (E - reference) + resolution (GG_BLUR_LINEAR), sigma = FWHM / 2.3548.
   Position: the energy-winner point in the crystal plane (a1, a2) moves by
   N(0, spatial_sigma); with keep_in_solid_limits points outside the crystal
   (|a| > half_width) are put just inside the edge (1e-6 half_width; the
   reference's 1 nm would round onto the edge in FP32); with truncated = 1 they
   are redrawn with the reference's corrected sigma instead.  The draws come
   from each history's own random stream; ARF training rows take the blurred
   energy's window.  All-zero descriptor = no blurring. */
#define GG_BLUR_NONE 0
#define GG_BLUR_GAUSSIAN 1
#define GG_BLUR_INVERSE_SQUARE 2
#define GG_BLUR_LINEAR 3
typedef struct {
  int32_t energy_method;        /* GG_BLUR_* */
  double energy_sigma;          /* MeV (Gaussian) */
  double energy_resolution;     /* FWHM / E at the reference energy */
  double energy_reference;      /* MeV */
  double energy_slope;          /* 1 / MeV (linear law) */
  int32_t spatial;              /* 0 off, 1 on */
  double spatial_sigma[2];      /* mm along a1, a2 */
  int32_t keep_in_solid_limits; /* clamp into the crystal */
  int32_t truncated;            /* redraw outside the crystal (truncated Gaussian) */
} gg_blur_desc;
int gg_spect_set_blur(gg_ctx *ctx, const gg_blur_desc *blur);

/* Free flight outside the heads (replaces GammaFreeFlightActor attached to the
   world with the heads as exclude_volumes: biasing/GateGammaFreeFlightOptn.cpp:34-83,
   GateGammaFreeFlightOptrActor.cpp, GateVBiasOptrActor.cpp:85-92,
   opengate/actors/biasingactors.py:247-300; the primary simulation of
   contrib/spect/spect_config.py:937-970).  Outside the heads photons do not
   interact: each flies straight to the nearest head entry and its weight is
   multiplied by exp(-optical depth) of the path (image voxels and world
   material); photons whose line misses every head stop, and so do photons
   at or below the energy or weight cutoff.  Inside the heads transport is
   analog.  Singles add their weight (and its history-by-history square)
   to the weighted projection read with gg_get_arf_projection; the counts of
   gg_get_projection stay zero.  Not together with the ARF detector. */
#define GG_FF_OFF 0
#define GG_FF_PRIMARY 1 /* GammaFreeFlightActor: no interaction outside the heads */
#define GG_FF_SCATTER 2 /* ScatterSplittingFreeFlightActor (below) */
#define GG_MAX_SPLITTING 4096
typedef struct {
  int32_t enabled;      /* GG_FF_OFF, GG_FF_PRIMARY or GG_FF_SCATTER */
  double weight_cutoff; /* photons with weight <= this stop (reference default -1) */
  double energy_cutoff; /* MeV, photons with energy <= this stop (reference default 0) */
  /* GG_FF_SCATTER (ScatterSplittingFreeFlightOptrActor, biasing/
     GateScatterSplittingFreeFlightOptrActor.cpp:200-420, GateScatterSplittingFreeFlightOptn.cpp:
     ApplyFinalStateBiasing_V1_PostStepDoIt): photons are tracked analog
     outside the heads and die when they enter one; each of their Compton
     scatterings (up to max_compton_level of them; the one after that kills
     the photon) and Rayleigh scatterings is re-sampled compton_splitting /
     rayleigh_splitting times from the state before it, each copy with
     1 / factor of the weight and its own random stream, and copies whose
     line reaches a head fly freely to it (angular acceptance: the heads) and
     are tracked there as in GG_FF_PRIMARY.  Factors are at most
     GG_MAX_SPLITTING.  A phantom pass whose copies overflow the head queue
     is repeated on fewer histories (results do not depend on the pass
     sizes). */
  int32_t compton_splitting;
  int32_t rayleigh_splitting;
  int32_t max_compton_level;
  /* angular acceptance, angle check (biasingactors.py generic_source_default_aa
     angle_tolerance_max): a photon (GG_FF_PRIMARY) or copy (GG_FF_SCATTER)
     whose line enters a head more than this many radians off the head's axis
     is dropped before its optical depth is computed, as the reference's
     free-flight recipes skip such directions at the source
     (contrib/spect/spect_config.py:937-970); <= 0: no angle check.  With the
     ARF detectors on (gg_spect_use_arf) free flight and the network combine:
     a photon reaching a head face is scored with its free-flight weight times
     the network's window weights. */
  double angle_tolerance_max;
} gg_ff_desc;
int gg_spect_set_free_flight(gg_ctx *ctx, const gg_ff_desc *ff);
int gg_spect_set_heads(gg_ctx *ctx, int32_t run, const double *frames);
int gg_spect_run(gg_ctx *ctx, uint64_t n_per_run, uint64_t seed, uint64_t first, const double *frames);
int gg_get_projection(gg_ctx *ctx, double *out, size_t n);

/* Singles list (replaces the "Singles" digi collection of DigitizerAdderActor
   and its ROOT ntuple: GateDigiCollection::FillToRoot,
   core/opengate_core/opengate_lib/digitizer/GateDigiCollection.cpp:114-128,
   written by GateDigiCollectionsRootManager; opengate/actors/digitizers.py:
   300-420).  gg_spect_record_singles(ctx, capacity) keeps, from the next
   gg_spect_run on, one gg_single per head single of the tracked heads (after
   the adder and the blurring, before the windows and the projection pixel
   test; network-scored ARF photons make no singles, as in the reference),
   in a device list of `capacity` records (0: off, the default).  Records are
   appended in completion order, not history order.  gg_spect_get_singles
   copies min(recorded, capacity, out_capacity) records to `out`, sets
   *n_recorded to all singles recorded since the list was last read or set
   (more than the list's capacity when it overflowed: those beyond were
   dropped) and empties the list.  Positions are the crystal-plane
   coordinates (a1, a2) of the head frame of gg_spect_set_heads, mm. */
typedef struct {
  uint64_t event_id; /* history index (the copies of scatter splitting keep their history's) */
  int32_t head;
  int32_t run;       /* gantry position */
  double energy;     /* MeV, after energy blurring */
  double a1, a2;     /* mm, along the head frame's e1 / e2, after spatial blurring */
  double weight;     /* free-flight weight (1 without free flight) */
} gg_single;
int gg_spect_record_singles(gg_ctx *ctx, uint64_t capacity);
int gg_spect_get_singles(gg_ctx *ctx, gg_single *out, uint64_t out_capacity, uint64_t *n_recorded);

/* ---- ARF surrogate ---------------------------------------------------------
   gg_arf_dataset replaces the ARF training-dataset simulation
   (GateARFTrainingDatasetActor, core/opengate_core/opengate_lib/
   GateARFTrainingDatasetActor.cpp:76-137, fed by
   contrib/spect/ge_discovery_nm670.py:994-1027): samples [first, first + n)
   of `sampling` are tracked through the head of gg_spect_setup (collimator,
   gap, crystal, energy windows) and give rows (E MeV, theta deg, phi deg, w)
   of float32, w = last window containing the crystal energy + 1, 0 = none
   (kept with probability 1 / russian_roulette).  Rows are in sample order;
   *n_rows = rows produced, the first min(*n_rows, capacity) are written. */
int gg_arf_dataset(gg_ctx *ctx, const gg_arf_sampling *sampling, uint64_t n, uint64_t seed, uint64_t first,
                   float *rows, uint64_t capacity, uint64_t *n_rows);

/* The ARF network (the garf model the reference's ARFActor loads from a .pth
   file, opengate/actors/arfactors.py:299-331): x = standardised (theta deg,
   phi deg, E MeV) -> 128 ReLU -> 128 ReLU -> 128 ReLU -> n_classes logits ->
   softmax; class 0 = no window, class k = window k.  Parameters are
   GG_ARF_N_PARAMS floats: W1[128][3], b1[128], W2[128][128], b2[128],
   W3[128][128], b3[128], W4[16][128] (rows >= n_classes zero), b4[16]
   (weights stored [out][in]).  Layers 2-4 run on the tensor cores in BF16
   with FP32 accumulation. */
#define GG_ARF_N_PARAMS 35600
typedef struct {
  int32_t n_classes;          /* energy windows + 1, <= 9 */
  float x_mean[3], x_std[3];  /* standardisation of (theta, phi, E) */
  double russian_roulette;    /* class-0 keep factor of the training rows; class 0 is re-weighted by it */
  double e_min, e_max;        /* trained energy domain, MeV */
  double theta_max_deg;       /* trained angular domain */
  double distance_to_crystal; /* mm from the collimator face to the projection plane */
} gg_arf_model;

typedef struct {
  uint64_t n_samples;   /* training photons (rows come from gg_arf_dataset of these samples) */
  uint64_t seed;        /* dataset seed (Philox stream 1) */
  uint64_t init_seed;   /* weight initialisation (He-uniform) */
  int32_t batch;        /* rows per Adam step, a multiple of 128, <= 65536 */
  int32_t epochs;
  float lr, beta1, beta2, eps;
  float lr_final;       /* learning rate decays exponentially from lr to lr_final over the steps (0: constant) */
} gg_arf_train_opts;

/* Generates the training rows of `sampling` on the device and trains the
   network with Adam (cross-entropy, mean over the batch); model_out gets the
   standardisation and domain (theta from sampling, energies from sampling),
   distance_to_crystal = collimator + gap + cover + half the crystal.  loss (epochs
   values, or NULL) = mean loss of each epoch.  The trained model becomes the
   context's ARF model. */
int gg_arf_train(gg_ctx *ctx, const gg_arf_sampling *sampling, const gg_arf_train_opts *opts,
                 gg_arf_model *model_out, double *loss);
/* Trains the network on caller-supplied rows instead of generating them: the
   garf training step (garf_train on the ROOT file the reference's
   ARFTrainingDatasetActor writes, GateARFTrainingDatasetActor.cpp:76-137)
   with this library's kernels.  rows[n_rows][4] = (E MeV, theta deg, phi
   deg, class), class 0 = no window (kept with probability 1 / rr), k =
   window k.  `domain` gives the trained energy range, theta_max_deg and
   russian_roulette (its other fields are ignored): the standardisation
   follows from them as for gg_arf_train.  opts->n_samples and opts->seed are
   not used. */
int gg_arf_train_rows(gg_ctx *ctx, const float *rows, uint64_t n_rows, const gg_arf_model *domain,
                      const gg_arf_train_opts *opts, gg_arf_model *model_out, double *loss);
/* Sets / reads the context's ARF model (params: GG_ARF_N_PARAMS floats). */
int gg_arf_set_model(gg_ctx *ctx, const gg_arf_model *model, const float *params);
int gg_arf_get_params(gg_ctx *ctx, float *params, size_t n);
/* Network outputs (softmax, before the class-0 re-weighting) of n rows
   (E, theta, phi, -) -> probs[n][n_classes]. */
int gg_arf_predict(gg_ctx *ctx, const float *rows, uint64_t n, float *probs);
/* Gradient of the mean cross-entropy of n rows (n a multiple of 128) at the
   current parameters, no update: grad[GG_ARF_N_PARAMS], *loss = mean loss. */
int gg_arf_gradient(gg_ctx *ctx, const float *rows, uint64_t n, float *grad, double *loss);

/* ARF detectors in the SPECT acquisition (GateARFActor::SteppingAction +
   ARFActor.apply, core/opengate_core/opengate_lib/GateARFActor.cpp:60-113,
   opengate/actors/arfactors.py:349-415).  With the ARF stage on, a photon
   that enters a head through the collimator face inside the model's energy
   / angle domain is scored by the network instead of being tracked: window
   weights p_k / (russian_roulette p_0 + sum_k>0 p_k) at the pixel where its
   line crosses the plane distance_to_crystal behind the face.  Photons
   entering elsewhere or outside the domain are tracked as before (counts in
   gg_get_projection); photons below every window are dropped.  The model
   needs n_windows + 1 classes.  gg_get_arf_projection returns the weights
   (and their history-by-history squares, or NULL) in the projection layout;
   gg_spect_setup zeroes them. */
int gg_spect_use_arf(gg_ctx *ctx, int32_t enable);
/* Device time of the last gg_run / gg_spect_run per SPECT stage (sums of
   CUDA-event intervals around the stage launches, ms); arf_ms holds the ARF
   stage, or with GG_FF_SCATTER the split and walk kernels of the copies. */
int gg_last_stage_ms(gg_ctx *ctx, double *phantom_ms, double *head_ms, double *arf_ms);
int gg_get_arf_projection(gg_ctx *ctx, double *counts, double *squared, size_t n);

/* ---- batched simulations (one set of launches for many simulations) ---------
   Many independent dose simulations - each with its own image, source,
   primaries, seed and DoseActor tally - sharing the tables and the world run
   through one persistent launch per batch of histories (the uneven
   simulations of a parameter study or a multi-patient queue; the reference
   runs them as separate Simulation objects, opengate/managers.py:1805).
   History i of simulation k uses the Philox stream (seed_k, i), so each
   simulation's images equal those of a gg_run of it alone (same seed,
   first history 0).  Sources: point/box/sphere/disc, iso/momentum/focused,
   mono/range (no spectra, voxel sources or acceptance boxes).
   gg_batch_setup replaces the context's volume, source and tally (upload the
   tables and set the world first); every simulation keeps its own majorant.  gg_batch_run simulates all primaries;
   gg_batch_capture records the launch sequence of one gg_batch_run in a CUDA
   graph and gg_batch_replay replays it (the same histories again, images
   accumulate: call gg_reset_tally between replays to repeat a step).
   gg_batch_autotune searches the launch configuration of the one persistent
   transport launch that takes the histories of all simulations from one
   device work counter: first blocks per SM x refill / interaction thresholds,
   then, at the best of those, the per-warp claim chunk x the batch length
   (histories per generate / transport / flush sequence).  Every point is
   timed as the median of three gg_batch_run calls; the fastest stays in the
   context (*best, may be NULL) and gg_batch_autotune_result reports the
   search (points timed, the winner's median / min / max); images are reset
   afterwards.
   gg_batch_get_image returns simulation `sim`'s image (its n voxels). */
typedef struct {
  gg_volume_desc volume;
  gg_source_desc source;
  uint64_t n_primaries;
  uint64_t seed;
} gg_sim_desc;

int gg_batch_setup(gg_ctx *ctx, const gg_sim_desc *sims, int32_t n_sims);
int gg_batch_run(gg_ctx *ctx);
int gg_batch_capture(gg_ctx *ctx);
int gg_batch_replay(gg_ctx *ctx);
int gg_batch_autotune(gg_ctx *ctx, gg_device_opts *best);
typedef struct {
  int32_t points;      /* configurations timed */
  int32_t repeats;     /* timings per configuration (median taken) */
  double median_ms;    /* the chosen configuration: median device time of gg_batch_run */
  double min_ms, max_ms;
  double default_median_ms; /* the configuration the context had before the search */
} gg_autotune_result;
int gg_batch_autotune_result(gg_ctx *ctx, gg_autotune_result *out);
int gg_batch_get_image(gg_ctx *ctx, int32_t sim, int32_t which, double *out, size_t n);

/* ---- dose run that allocates no device memory ------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they work: cudaMalloc/cudaFree synchronise the whole device (a caller
 * keeping other streams busy, such as an optimisation loop calling the dose
 * engine many times, cannot afford that) and a caller whose device memory is
 * already handed out by its own pool may have none left for another
 * allocator.  The run uses the same kernels as gg_run; every scratch buffer
 * lives in one static device array of GG_NOALLOC_SCRATCH_BYTES, which each GPU
 * that loads the library reserves until the process exits.
 *
 * Inputs are the host descriptors of gg_upload_tables / gg_upload_volume /
 * gg_set_world / gg_set_source; outputs are device pointers owned by the
 * caller: d_edep (and d_edep2, or NULL to skip the squared image), n voxels
 * of float64 each, overwritten with the edep / edep-squared images of
 * histories [first_history, first_history + n_histories).  FP32 transport,
 * batches of GG_NOALLOC_BATCH histories: the images equal those of gg_run
 * with the same seed, histories and batch size.  Work runs on `stream`
 * (cudaStream_t, NULL = legacy default stream) and is complete on return.
 * counters (host, GG_N_COUNTERS slots) may be NULL; on error a message is
 * written to err (err_len bytes, NUL-terminated).
 *
 * Sizes beyond the GG_NOALLOC_MAX_* limits, and voxel (activity image)
 * sources, are rejected with GG_ERR_ARG.
 * All calls share the scratch array: each call clears the parts that must
 * start at zero, and calls whose GPU work overlaps (other threads or
 * unordered streams) race on it - serialise them.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture on the device.
 */
#define GG_NOALLOC_SCRATCH_BYTES (32u << 20)
#define GG_NOALLOC_MAX_VOXELS (1u << 20)
#define GG_NOALLOC_BATCH 65536
#define GG_NOALLOC_MAX_ENERGIES 512
#define GG_NOALLOC_MAX_COMPOSITIONS 16
#define GG_NOALLOC_MAX_RAYLEIGH 1024
#define GG_NOALLOC_MAX_MATERIALS 4096
#define GG_NOALLOC_MAX_SPECTRUM 1024
#define GG_NOALLOC_MAX_ACCEPT 16
int gg_dose_run_noalloc(int32_t device, void *stream, const gg_tables_desc *tables, const gg_volume_desc *volume,
                        const gg_world_desc *world, const gg_source_desc *source, uint64_t n_histories,
                        uint64_t seed, uint64_t first_history, double *d_edep, double *d_edep2,
                        uint64_t *counters, char *err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* GATE_GPU_H */
