// Ozaki-split FP64 contraction on the FP8 (e4m3) tensor cores of sm_103a.
#pragma once

#include <vector>

#include "common.cuh"

namespace hsdla {

constexpr int kOzMaxSlices = 12;
// 11 digits (4 + 5*10 = 54 bits per value, 66 digit products) keep the relative error
// of H and S near 1e-15 on the FLAPW workloads; 10 digits land at ~1e-13.
constexpr int kOzDefaultSlices = 11;

struct OzakiPlan {
    int num_slices = 0;          // digit slices per operand
    double target = 1e-13;
    int *d_error = nullptr;      // device error word (bounded waits)
};

// Inputs of one k-point: C = [A_a; B_a] (K = 2 L a rows, G columns, ld K),
// per-type Hermitian T blocks (2L x 2L each, column-major, concatenated),
// S row weights w (K), FP64 workspace X (K x G, ld K).
struct OzakiInputs {
    const double2 *C;
    const double2 *Tfull;
    const double *w;
    const int32_t *atom_type;    // host array [na]
    double2 *X;
    int64_t twoL, na, nt, G;
    cudaEvent_t ev_dom0 = nullptr, ev_dom1 = nullptr;   // recorded around the S/H launch when set
    // Per-type T application (atoms share their rotation): phase-free rows M ((2L nt) x G, ld 2L nt),
    // FP64 workspace Z of the same shape, and the data the phase expansion X_a = phase_a Z_t needs.
    const double2 *M = nullptr;
    double2 *Z = nullptr;
    const DevSystem *sys = nullptr;
    const DevKpoint *kp = nullptr;
};

// ---- k-point groups (prepared once per plan, run per execution; runs are graph-capturable)
struct OzKBufs {
    double2 *CX = nullptr;   // FP64 C of the k-point; reused for X once C is sliced (K x G, ld K)
    double2 *M = nullptr;    // per-type rows M (2L nt x G), hoisted T application only
    double2 *Z = nullptr;    // per-type products Z (2L nt x G), hoisted T application only
    int64_t G = 0;
    double2 *PS = nullptr;   // structure-factor form: per-type products (G x G, ld G), type
    double2 *PH = nullptr;   // slot b of a combine batch at + b pstride
    int64_t pstride = 0;
};
struct OzGroupDesc {
    int64_t twoL = 0, na = 0, nt = 0;
    bool hoist = false;
    const double *w = nullptr;             // S row weights (K)
    const double2 *Tfull = nullptr;        // per-type 2L x 2L blocks
    const int32_t *atom_type = nullptr;    // host [na]
    int panels = 1;                        // atom panels the contraction index is streamed in
    bool sf = false;                       // structure-factor form (requires hoist)
    const double *wt = nullptr;            // its per-type S weights [nt][2L]
    const double2 *sf_tab = nullptr;       // its structure factors
    int tbatch = 1;                        // its types per combine batch (product slots)
};
struct OzGroup;
// scratch: rewritten by every run (may be shared by the groups of a plan); persist: owned by
// the group for its lifetime (T digits, job tables, schedules)
// Panels: the atoms split into `panels` contiguous ranges; only one panel's digit planes are
// resident at a time (the scratch shrinks accordingly), the S/H products accumulate over panels.
int64_t ozaki_group_bytes(int s, int64_t twoL, int64_t na, int64_t nt, const std::vector<int64_t> &G, int panels,
                          bool hoist, bool sf);
int64_t ozaki_group_persist_bytes(int s, int64_t twoL, int64_t na, int64_t nt, const std::vector<int64_t> &G,
                                  int panels);
int ozaki_group_prepare(OzakiPlan &oz, const OzGroupDesc &d, const std::vector<OzKBufs> &kb, void *ws,
                        void *persist, cudaStream_t st, OzGroup **out);
void ozaki_group_set_outputs(OzGroup *g, double2 *const *S, double2 *const *H, const int64_t *ld);
// Structure-factor form: the group's combine table (outputs of this run, per-type products).
void ozaki_group_set_sf(OzGroup *g, const SfTab &t);
// Structure-factor form: the first type of the group's last combine (types [t0, nt), adding to
// S and H unless t0 = 0): what ozaki_group_run leaves to its caller with defer_last_combine.
int ozaki_group_last_combine(const OzGroup *g);
// Enqueues the group's launches (slices, T application, phases, S/H products); no host sync.
// ev: event pairs recorded around the S/H product launches (one pair, or one per type in the
// structure-factor form; nev events, may be 0).  defer_last_combine: the structure-factor form's
// last combine batch is left to the caller.  ev_t: event pairs recorded around the T-application
// launches (one pair, or one per atom panel when each panel applies T itself; nev_t events, may
// be 0; plain records, so not for a run under graph capture).  host_out (streamable groups only,
// see ozaki_group_streamable; not under graph capture): the combine table whose outputs are the
// caller's page-locked host H and S; the S/H products then run in column blocks and each block is
// combined into those outputs while the next block's products run (the whole combine is done
// when the call's work on st completes; defer_last_combine does not apply).
int ozaki_group_run(OzGroup *g, const DevSystem &sys, const KTable &ktab, cudaStream_t st, const cudaEvent_t *ev,
                    int nev, int *launches, bool defer_last_combine = false, const cudaEvent_t *ev_t = nullptr,
                    int nev_t = 0, const SfTab *host_out = nullptr);
// A structure-factor group whose host outputs can be written in column blocks while its products
// run (pair tiles, every type in one combine batch, at least two blocks; HSDLA_STREAM_OUTPUT=0
// turns it off), and its block count.
bool ozaki_group_streamable(const OzGroup *g);
int ozaki_group_output_blocks(const OzGroup *g);
// Event pairs ozaki_group_run records around the group's T application (see ev_t).
int ozaki_group_tapply_events(const OzGroup *g);
void ozaki_group_destroy(OzGroup *g);
// The structure-factor form's S/H tile configuration on CTA-pair tiles: halves 1 (256 x 256
// accumulators) or 2 (two 256 x 128 halves), merged 1 (adjacent digit diagonals share exact
// accumulation units) or 0.  Tunable: a structure-factor group on pair tiles.
bool ozaki_group_tunable(const OzGroup *g);
void ozaki_group_tiles(const OzGroup *g, int *halves, int *merged);
void ozaki_group_set_tiles(OzGroup *g, int halves, int merged);
// Times the first type's S/H launch in each configuration on the digit planes of a completed
// run and keeps the fastest (ms_best: its time).
int ozaki_group_tune_tiles(OzGroup *g, cudaStream_t st, float *ms_best);

int ozaki_plan_init(OzakiPlan &oz, int num_slices, double target);
void ozaki_plan_release(OzakiPlan &oz);
int64_t ozaki_pipeline_workspace(int s, int64_t twoL, int64_t na, int64_t nt, int64_t G);
int64_t ozaki_herkx_workspace(int s, int64_t K, int64_t n);
// S = C^H diag(w) C and H = C^H (T C) (lower triangles) with the T application emulated too.
int ozaki_pipeline(OzakiPlan &oz, const OzakiInputs &in, double2 *S, double2 *H, int64_t ldo, void *ws,
                   cudaStream_t st, int *launches);
// OUT = P^H diag(w) Q, lower triangle (standalone component).
int ozaki_herkx(OzakiPlan &oz, const double2 *P, int64_t ldp, const double2 *Q, int64_t ldq, const double *w,
                int64_t K, int64_t n, double2 *out, int64_t ldo, void *ws, cudaStream_t st, int *launches);
int ozaki_check_device_error(OzakiPlan &oz);
// Lets one bounded wait expire on purpose (0: an mbarrier nothing arrives on, 1: a lockstep slot
// that never advances) after budget_cycles; returns the status the host reads (HSDLA_ERR_TIMEOUT).
int ozaki_wait_selftest(OzakiPlan &oz, int which, long long budget_cycles, cudaStream_t st);
const char *ozaki_last_error();

}  // namespace hsdla
