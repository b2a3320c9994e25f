// ss4d_kernels.cuh — kernel-side declarations shared by the kernel
// translation units and the host orchestration (ss4d_api.cu).
#pragma once

#include "ss4d_common.cuh"

namespace ss4d {

struct GPtrs8 {
    double *p[8];
};
struct CPtrs8 {
    const double *p[8];
};

// ---- natural-layout, reference-order kernels (ss4d_kernels_ref.cu) -------
long long interior_blocks(const Geo &g);
long long resid_blocks(const Geo &g); // partials of the residual passes
void launch_reflect(const Geo &g, double *u, cudaStream_t st);
void launch_presmooth_half(const Geo &g, double *v, const double *prev, double c, double omega, int colour,
                           cudaStream_t st);
void launch_presmooth_explicit(const Geo &g, double *v, const double *prev, double coeff, cudaStream_t st);
// normalised Gaussian taps w[0..R] of one axis (ss4d_gaussian_smooth)
struct GaussWeights {
    double w[SS4D_GAUSS_MAX_RADIUS + 1];
    int R;
};
void launch_gauss_axis(const Geo &g, int axis, const double *in, double *out, const GaussWeights &W,
                       cudaStream_t st);
void launch_presmooth_resid(const Geo &g, const double *v, const double *prev, double c, double h4, double *partial,
                            cudaStream_t st);
void launch_gfaces(const Geo &g, const double *i0, const double *ithr, GPtrs8 gout, double h, double K, double theta,
                   double rho, cudaStream_t st);
void launch_coef_ref(const Geo &g, const double *u, CPtrs8 gin, int has_g, GPtrs8 coef, double h, double eps2,
                     cudaStream_t st);
void launch_sor_half_ref(const Geo &g, double *u, const double *prev, CPtrs8 a, double c, double omega, int colour,
                         cudaStream_t st);
void launch_sor_resid_ref(const Geo &g, const double *u, const double *prev, CPtrs8 a, double c, double h4,
                          double *partial, cudaStream_t st);
// sums n partials into *out; may use partial[n .. n + 1024) (returns the launches)
int launch_reduce_sum(double *partial, long long n, double *out, cudaStream_t st);
void launch_l2(const Geo &g, const double *a, const double *b, double h4, double *partial, int nblk, cudaStream_t st);
void launch_mass(const Geo &g, const double *a, double h4, double *partial, int nblk, cudaStream_t st);
void launch_mcf_field(const Geo &g, double *u, double h, double t, int ghosts_only, cudaStream_t st);
void launch_rescale_balls(const Geo &g, double *v, const int *frame_first, const int *frame_count, const double *bx,
                          const double *by, const double *bz, double R, cudaStream_t st);
void launch_mask_zero(const Geo &g, double *v, const double *Mmask, cudaStream_t st);
// one frame <-> file bytes: img_out != null: bytes_in -> frame l of img_out;
// else frame l of img_in -> bytes_out (mode 0 scaled, 1 mask)
void launch_frame_bytes(const Geo &g, double *img_out, const double *img_in, int l, int mode, const uint8_t *bytes_in,
                        uint8_t *bytes_out, cudaStream_t st);
// initial segmentation (segmentation4D.c:876-1018, 1106-1147)
void launch_ball_min_max(const Geo &g, const double *v, int l, double cx, double cy, double cz, double R, double *out2,
                         cudaStream_t st);
void launch_local_threshold(const Geo &g, const double *in, double *thr, const int *frame_first, const int *frame_count,
                            const double *bx, const double *by, const double *bz, double R, double alpha, double beta,
                            const double *minmax, cudaStream_t st);
void launch_generate_segm(const Geo &g, double *u, double *Mmask, const int *frame_first, const int *frame_count,
                          const double *bx, const double *by, const double *bz, double R, cudaStream_t st);
// interior min, max and min + level (max - min) of u into out3; partial needs
// 4096 doubles (returns the launches)
int launch_minmax(const Geo &g, const double *u, double *partial, double level, double *out3, cudaStream_t st);
void launch_threshold(const Geo &g, const double *u, const double *level_dev, double level, uint8_t *mask,
                      cudaStream_t st);

// ---- colour-split fast forms (ss4d_kernels_fast.cu) ------------------------

// Device-resident loop state of one SOR solve.  The controller kernel is its
// only writer during the loop; sweeps read it to pick their buffers.
struct LoopState {
    int z;           // current iteration (fast FP64 form); inner sweeps (mixed)
    int stop;        // 1 once the loop has ended
    int status;      // ss4d_status
    int mode;        // mixed form: 0 refine, 1 start round, 2 inner sweep
    int refinements; // mixed form: FP64 residual/refinement passes done
    int round_z;     // mixed form: sweeps in the current round
    int dsrc;        // mixed form: ping-pong index of the current red correction
    int final_red;   // red buffer holding the result once the loop stopped
    int bodies;      // loop bodies the controller has run
    int keep;        // mixed form: the next round starts from the correction already in place
    int warm;        // mixed form: this step's first correction came from the learned predictor
    int near;        // 1 once a stop test saw |R - tol| <= near_band
    int pre;         // mixed form: the next refinement pass's residual is in rpre (formed by the
                     // assembly, which also applied the start correction); cleared by that pass
    int proj;        // mixed form: the first round starts from the projection onto the previous
                     // steps' changes (ss4d_project.cu)
    int spec;        // mixed form: pause the loop when a round ends, before its refinement pass
                     // (the host-array step downloads the round's result meanwhile)
    int paused;      // set by the controller when it paused the loop (spec); the refinement clears it
    double R;        // last FP64 residual (sum r^2 h^4)
    double R_first;  // FP64 residual after iteration 1 (fast) / initial (mixed)
    double Rd;       // mixed form: last FP32 correction residual
    double target;   // mixed form: round target for Rd
};

// Scalars the fast kernels read from device memory so that one captured
// graph serves every call of a solver.
struct DevParams {
    double c;        // tau / h^2
    double omega;    // omega_c
    double h4;       // h^4
    double tol;      // gsTol
    int maxit;       // maxNoGSIteration
    int pad_;
    // |R - tol| below this band: a serial sum of the same terms (the
    // reference's order) could have decided the stop test the other way
    double near_band;
};

// Buffers of the colour-split FP64 form.
struct SplitBufs {
    double *R[2];       // red u, ping-pong (all cells incl. ghosts)
    double *Bk;         // black u (all cells incl. ghosts)
    double *P[2];       // prev (per colour)
    double *coef[2];    // per colour, record t (coef_at(t, f, 10)): f < 8: c*a_f (f = e,w,n,s,t,b,fw,bw),
                        // f = 8: diag, f = 9: omega/diag;  10 * ct doubles
    // mixed form, records of the FP32 sweeps, per colour and target t: the
    // scale s = sum_f c*a_f (coefs[t], FP32) and the fractions c*a_f / s as
    // eight 16-bit fixed-point numbers (coefq[t], faces in record order);
    // 20 bytes per target (store_coef16 / load_coef16 in ss4d_sweep.cuh)
    uint4 *coefq[2];
    float *coefs[2];
    float *dR[2];       // mixed: red correction, ping-pong
    float *dB;          // mixed: black correction
    float *r32[2];      // mixed: FP64 residual rounded to FP32, per colour
    double *partial[2]; // per-block residual partials of the red [0] / black [1] kernels
    // assembly: per voxel v and axis d, the quantities of the face between v
    // and v + e_d (natural layout): |grad u|_eps and g/|grad u|_eps
    double *fn[4];
    double *fq[4];
    // mixed form's float-float assembly (ss4d_assemble_ff.cu): per voxel v and
    // axis a the forward difference u(v + e_a) - u(v) as two floats
    double *fd[4];
    // mixed form, first refinement pass of a segmentation step: its FP64
    // residual per target, formed by the coefficient kernel (split layout)
    double *rpre[2];
};

struct SweepCfg {
    int threads;   // threads per block (256)
    int XT;        // threads along x in a tile (power of two)
    int TJ;        // rows (j) per tile
    int KB;        // k-block depth of the tile order
    int nXC;       // x chunks per row
    int nJG;       // j groups
    int nKB;       // k blocks
    long long ntiles;  // below 2^31 (fewer than the voxels)
    int grid;      // persistent grid (blocks)
    FastDiv dXC, dJG, dKB, dNT; // nXC, nJG, KB, nt for the tile coordinates
};

SweepCfg make_sweep_cfg(const Geo &g, const Split &s, int sm_count, int kb);

void launch_assemble(const Geo &g, const Split &s, const double *u, CPtrs8 gin, int has_g, const ss4d_params &p,
                     SplitBufs b, int want32, cudaStream_t st);
void launch_pack(const Geo &g, const Split &s, const double *u, const double *prev, SplitBufs b, cudaStream_t st);
// mixed form: the same coefficient records from float-float arithmetic (3
// kernels); with pack the first of them also makes launch_pack's copies of u
// with prev = u
// (kblock: block order of the faces and coefficient kernels, as in
// launch_assemble_ff_faces_range)
void launch_assemble_ff(const Geo &g, const Split &s, const double *u, CPtrs8 gin, int has_g, const ss4d_params &p,
                        SplitBufs b, int pack, int sm_count, cudaStream_t st, int pre = 0, int kblock = 0);
// the same in parts: first differences of padded frames [l0, l1), then the
// faces and voxel coefficients (after the differences of every frame)
void launch_fdiff_range(const Geo &g, const double *u, SplitBufs b, int l0, int l1, int sm_count, cudaStream_t st);
// the same plus launch_pack_range's copies of those frames with prev = u;
// with pre > 0 the interior of the u copies also receives the first
// refinement pass's start correction (pre 2: the one in dR[0] / dB; pre 1:
// zero, added as the pass adds it)
void launch_fdiff_pack_range(const Geo &g, const Split &s, const double *u, SplitBufs b, int l0, int l1, int sm_count,
                             cudaStream_t st, int pre = 0);
void launch_assemble_ff_faces(const Geo &g, const Split &s, CPtrs8 gin, int has_g, const ss4d_params &p, SplitBufs b,
                              cudaStream_t st, int pre = 0, int kblock = 0);
// faces of the frames [f0, f1) of the extended box (0 .. nt; they need the
// first differences of frames f0-1 .. f1) and coefficients of the interior
// frames [v0, v1) (they need the faces of frames v0-1 .. v1-1); empty ranges
// launch nothing.  With pre the coefficient kernel also forms the first
// refinement pass's residual into rpre (it needs the corrected split copies
// of u of frames v0-1 .. v1).  kblock orders the blocks of both kernels:
// 0 frame by frame (all planes of a frame, then the next frame), n >= 1 in
// blocks of n planes (those planes of every frame in turn, then the next n
// planes), which keeps a frame's neighbours in the next frame and the next
// plane close in time; results do not depend on it
void launch_assemble_ff_faces_range(const Geo &g, const Split &s, CPtrs8 gin, int has_g, const ss4d_params &p,
                                    SplitBufs b, int f0, int f1, int v0, int v1, cudaStream_t st, int pre = 0,
                                    int kblock = 0);
// frame ranges: padded frames [l0, l1) for the pack, interior frames
// [l0, l1) (1 <= l0 < l1 <= lMax-1) for the unpack and the rescale
void launch_pack_range(const Geo &g, const Split &s, const double *u, const double *prev, SplitBufs b, int l0, int l1,
                       cudaStream_t st);
// what k_unpack writes: u and the extrapolation history (UNPACK_ALL), only u
// of a loop paused before its last refinement pass (UNPACK_PAUSED: the split u
// plus the round's correction), only the history (UNPACK_HISTORY)
enum { UNPACK_ALL = 0, UNPACK_PAUSED = 1, UNPACK_HISTORY = 2 };
void launch_unpack_range(const Geo &g, const Split &s, SplitBufs b, const LoopState *state, double *u, cudaStream_t st,
                         int terms, int keep, float *const *hist, int l0, int l1, int what = UNPACK_ALL);
void launch_mask_zero_range(const Geo &g, double *v, const double *Mmask, int l0, int l1, cudaStream_t st);
void launch_rescale_balls_range(const Geo &g, double *v, const int *frame_first, const int *frame_count,
                                const double *bx, const double *by, const double *bz, double R, int l0, int l1,
                                cudaStream_t st);

// the mixed form's edge detector in float-float arithmetic (ss4d_front_ff.cu);
// float2 arrays hold (high, low) pairs in the natural layout
struct FFc {
    float h, l; // a constant split on the host
};
FFc split_ff(double v);
void launch_to_ff(const Geo &g, const double *a, float2 *out, cudaStream_t st);
void launch_from_ff(const Geo &g, const float2 *v, double *out, cudaStream_t st); // interior only
void launch_presmooth_half_ff(const Geo &g, float2 *v, const float2 *prev, double c, double omega, int colour,
                              cudaStream_t st);
long long front_resid_blocks(const Geo &g); // partials of launch_presmooth_resid_ff
void launch_presmooth_resid_ff(const Geo &g, const float2 *v, const float2 *prev, double c, double h4,
                               double *partial, cudaStream_t st);
void launch_gfaces_ff(const Geo &g, const float2 *i0, const float2 *ithr, GPtrs8 gout, double h, double K,
                      double theta, double rho, cudaStream_t st);
void launch_pack_coef(const Geo &g, const Split &s, CPtrs8 a, const ss4d_params &p, SplitBufs b, int want32,
                      cudaStream_t st);
// terms/keep/hist: the mixed form's extrapolated start (k_unpack); hist = {h1 red, h1 black, h2 red, h2 black}
void launch_unpack(const Geo &g, const Split &s, SplitBufs b, const LoopState *state, double *u, cudaStream_t st,
                   int terms = 0, int keep = 0, float *const *hist = nullptr);
void launch_loop_init(LoopState *state, int mode, cudaStream_t st, int pre = 0, int spec = 0);
void launch_sweep64(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                    LoopState *state, cudaStream_t st);
void launch_advance(LoopState *state, cudaStream_t st);
void launch_ctrl64(SplitBufs b, int nparts, const DevParams *dp, LoopState *state, unsigned long long cond_handle,
                   int use_cond, cudaStream_t st);

// mixed precision
void launch_refine(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                   LoopState *state, cudaStream_t st);
void launch_zero_delta(const Split &s, SplitBufs b, LoopState *state, cudaStream_t st);
void launch_sweep32(const Geo &g, const Split &s, const SweepCfg &cfg, int colour, SplitBufs b, const DevParams *dp,
                    LoopState *state, int start_mode, cudaStream_t st);
void launch_ctrl_mixed(SplitBufs b, int nparts, const DevParams *dp, LoopState *state, unsigned long long cond_handle,
                       int use_cond, cudaStream_t st);

int max_blocks_sweep64();
int max_blocks_sweep32();

// sets the text ss4d_last_error() returns (ss4d_api.cu)
void set_error_text(const char *msg);

// ---- learned warm start, solver side (ss4d_ws.cu) --------------------------
void launch_ws_features(const Geo &g, const Split &sp, SplitBufs b, const double *i0, CPtrs8 gin,
                        const LoopState *st, const DevParams *dp, void *x0, cudaStream_t s);
void launch_ws_apply(const Geo &g, const Split &sp, SplitBufs b, const float *y, const LoopState *st,
                     const DevParams *dp, cudaStream_t s);
void launch_ws_check_decide(const Geo &g, const Split &sp, const SweepCfg &cfg, SplitBufs b, LoopState *st,
                            const DevParams *dp, cudaStream_t s);

// ---- a handle's colour-split machinery, for the batched solver ------------
// (ss4d_api.cu; every call issues work on the handle's stream)
struct SolverView {
    Geo g;
    Split sp;
    SweepCfg cfg;
    SplitBufs b;
};
// the first round's start from the previous steps' changes (ss4d_project.cu):
// hist = the extrapolation history arrays (h1 red, h1 black, h2 red, h2 black),
// m = 2 or 3 vectors, part = 18 * cfg.grid doubles, c = 3 floats
void launch_projection(const Geo &g, const Split &sp, const SweepCfg &cfg, SplitBufs b, float *const *hist, int m,
                       double *part, float *c, LoopState *st, int sm_count, cudaStream_t s);
SweepCfg make_sweep_cfg_xt(const Geo &g, const Split &s, int sm_count, int kb, int xt);
// tiles of the kernels that give each thread two adjacent targets of a row
// (the FP32 sweep, the projection's products): cfg's row chunks of cfg.XT
// targets taken by cfg.XT / 2 threads, twice the rows per tile
SweepCfg make_pair_cfg(const Geo &g, const Split &s, const SweepCfg &cfg);
ss4d_status solver_view(ss4d_solver *s, SolverView *out);      // allocates the FP64 split buffers
ss4d_status solver_set_shape(ss4d_solver *s, int xt, int kb);  // tile width (threads along x) and k-block depth
// assemble the coefficients of u and pack u (= prev) into the split buffers;
// with pre_out (mixed form) the assembly also forms the first refinement
// pass (its start correction added, its residual in rpre) and *pre_out gets
// the LoopState.pre value the loop must start with (0 without pre_out)
ss4d_status solver_prepare_step(ss4d_solver *s, const ss4d_params *p, double *d_u, const double *const d_g[8],
                                int *pre_out = nullptr);
// unpack the red buffer state->final_red and black into the interior of u
ss4d_status solver_finish_step(ss4d_solver *s, const LoopState *d_state, double *d_u);
// the first round's projected start (ss4d_solver_set_projection) for a loop
// whose state is *d_state, when the step's assembly applied the
// extrapolation (pre == 2 from solver_prepare_step); nothing otherwise
ss4d_status solver_project_start(ss4d_solver *s, int pre, LoopState *d_state);
// device time of `iters` (black + red) FP64 sweep pairs with the current shape
ss4d_status solver_time_sweeps(ss4d_solver *s, const ss4d_params *p, int iters, float *ms);
int solver_sm_count(const ss4d_solver *s);

} // namespace ss4d
