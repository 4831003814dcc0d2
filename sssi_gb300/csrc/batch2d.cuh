// Batched 2D CPML step: many independent propagations ("shots"), each with
// its own grid, model, start step and length, advanced by one persistent
// launch per time step.  The tiled kernel of tile2d.cuh generalised so that a
// CTA's tiles may belong to different shots.
//
// Per-shot state and per-step hooks live in a device-resident array of
// ShotDesc.  A launch advances every active shot by one step; its batch step is
// a device-resident base plus a per-launch offset, so a captured run of K steps
// (offsets 0..K-1, then base += K) replays as a CUDA graph.  Consecutive steps
// are launched with programmatic stream serialization: the next step's blocks
// set up and fetch their work lists while the previous step drains.
#pragma once

#include "tile2d.cuh"

namespace sssi {

// Per-shot fields the tile code reads; copied to shared memory once per tile.
// The first 16 bytes are what the thread that prepares a tile needs (it keeps
// them in registers).
template <typename T>
struct alignas(16) ShotTail {
    using M = typename MemVar<T>::type;
    int t_start;     // batch step of the shot's first step
    int nt;          // steps of the shot
    unsigned sched;  // derived on upload (sched_word): reverse, which hooks are set, stride
    int oz;          // row offset of the interior in the padded fields
    T* field[2];  // interior origin of field k; field (t_local & 1) is current at local step t_local
    const T* zb;
    const T* zbm1;
    M* zphi[2];
    M* zpsi;
    const T* xb;
    const T* xbm1;
    M* xphi[2];
    M* xpsi;
    int64_t ldp;
    int nz, nx, nB, ntz, ntx;
    int reverse;  // time index tau = nt-1-t_local when set, else t_local
    int nsrc;
    int src_iz[kMaxPointSources];
    int src_ix[kMaxPointSources];
    const T* src_wavelet;  // nsrc x nt, indexed by tau
    const T* src_row;      // nx x nt: injected on row 0 at tau
    const T* src_dense;    // slices of nz x nx for tau = dense_t0, dense_t0+1, ...
    T* rec;                // nx x nt: row 0 after the step at tau
    T* snap;               // slices of nz x nx for tau = snap_t0, ...
    int dense_t0;
    int snap_t0;
    // RTM, forward shot: the field is stored in FP16 every `stride` steps with
    // one power-of-two scale per 32 x 32 block of cells (block (bz, bx) =
    // rows 32 bz .. 32 bz + 31, columns 32 bx .. 32 bx + 31; index bz + bx * nbz,
    // nbz = ceil(nz / 32), nblk blocks): at tau % stride == 0 each block's max
    // |field| goes to amax[(tau/stride) * nblk + block]; at (tau-1) % stride == 0
    // the current field (the result of step tau-1) is stored at
    // pack + ((tau-1)/stride) * nz*nx, scaled by its block's scale.
    int stride;
    unsigned* amax;
    __half* pack;
    float* perr;    // with pack: each cell's FP16 rounding error, added to its next stored value (nz x nx)
    float2* s2acc;  // when set: at tau % stride == 0, s2acc += field^2 (compensated), from the FP32 field
    // RTM, reverse shot: at tau % stride == 0 image against the stored forward
    // field, unscaled with the block maxima the forward shot recorded (the
    // illumination sum only when img_s22 is set)
    const __half* img_f16;     // stored forward fields (as written by pack)
    const unsigned* img_amax;  // their block maxima
    float2* img_m2;         // compensated FP32 sums
    float2* img_s22;
    const double* img_f64;  // FP64: forward field of every step, nz x nx x nt
    double* img_m;
    double* img_s2;
    // Residual pair (sched & kSchedPair, FP32 only): the shot advances two
    // fields in one tile, the field P of the model it was added with (the
    // migration model of an RTM shot) and the residual D = Q - P, where Q is
    // the field of a second model (the true model).  D is stored dcol columns
    // to the right of P in the same buffers and P's low part (P = hi + lo)
    // 2 dcol columns on ((v dt)^2 holds P's and, dcol columns on, the
    // difference Q's minus P's); the band factors b_Q - b_P follow P's b and
    // D's memory variables follow P's, zoff / xoff entries on.  rec_d receives
    // D's row 0.
    T* rec_d;
    int dcol;
    // the shot's status word: the step sets it to SSSI_ERR_UNSTABLE when a
    // value of row 0 (the receiver row) is not finite
    int* status;
};

// Per-tile work flags.  kBandZ, kBandX and point sources inside the tile do
// not change between steps and come with the work item; the rest are worked
// out per step by the thread that prepares the tile.
constexpr unsigned kBandZ = 1u;   // the z stencil of some cell reaches the damped band
constexpr unsigned kBandX = 2u;   // the x stencil of some cell reaches a damped band
constexpr unsigned kSource = 4u;  // something is injected into the tile at this step
constexpr unsigned kRare = 8u;    // snapshot / FP16 pack / max / imaging output at this step
constexpr unsigned kAmax = 16u;   // the step's max |field| is wanted

// kBandZ / kBandX of the tile at (z0, x0) of an nz x nx grid with nB-cell bands
// (bottom, left, right), stencil order N, tiles of TZ x TX cells.
__host__ __device__ inline unsigned tile_band_flags(int N, int TZ, int TX, int nz, int nx, int nB, int z0, int x0) {
    unsigned f = 0u;
    if (nB > 0 && z0 + TZ + N - 1 > nz - nB) f |= kBandZ;
    if (nB > 0 && (x0 - N < nB || x0 + TX + N - 2 >= nx - nB)) f |= kBandX;
    return f;
}

// ShotTail::sched: bit 0 reverse, bits 1-7 the hooks that are set, bit 8 a
// residual pair, the stride from bit 9 on.
constexpr unsigned kSchedReverse = 1u, kSchedDense = 2u, kSchedRow = 4u, kSchedSnap = 8u, kSchedImg64 = 16u,
                   kSchedAmax = 32u, kSchedPack = 64u, kSchedImg16 = 128u, kSchedPair = 256u;
constexpr int kSchedStrideShift = 9;
// hooks written by rare_outputs (or the block maxima) on some steps
constexpr unsigned kSchedRareOut = kSchedSnap | kSchedImg64 | kSchedAmax | kSchedPack | kSchedImg16;
template <typename T>
inline unsigned sched_word(const ShotTail<T>& d) {
    unsigned w = d.reverse ? kSchedReverse : 0u;
    if (d.src_dense) w |= kSchedDense;
    if (d.src_row) w |= kSchedRow;
    if (d.snap) w |= kSchedSnap;
    if (d.img_f64) w |= kSchedImg64;
    if (d.amax) w |= kSchedAmax;
    if (d.pack || d.s2acc) w |= kSchedPack;
    if (d.img_f16) w |= kSchedImg16;
    if (d.dcol > 0) w |= kSchedPair;
    return w | ((unsigned)(d.stride > 0 ? d.stride : 1) << kSchedStrideShift);
}

// A work item: shot k (< 2^24) with the tile's step-independent flags in the
// top byte; the tile's first row z0 and first column x0 (a shot's tiles may
// start above row 0 and left of column 0, see Batch2d::schedule) as
// (z0 + kZBias) / 4 and (x0 + kXBias) / 2, 16 bits each.
constexpr int kZBias = 128, kXBias = 64;  // z0 >= -(TZ - 1) of the deepest tile shape
constexpr int kMaxTileRow = 4 * 0xffff - kZBias;  // largest z0
constexpr int kMaxTileCol = 2 * 0xffff - kXBias;  // largest x0
__host__ __device__ inline int2 pack_work_item(int k, unsigned flags, int z0, int x0) {
    return make_int2((int)((unsigned)k | (flags << 24)),
                     (int)((unsigned)((z0 + kZBias) >> 2) | ((unsigned)((x0 + kXBias) >> 1) << 16)));
}
__host__ __device__ inline int work_item_z0(int2 item) { return (int)(item.y & 0xffff) * 4 - kZBias; }
__host__ __device__ inline int work_item_x0(int2 item) { return (int)((unsigned)item.y >> 16) * 2 - kXBias; }

template <typename T>
struct alignas(128) ShotDesc {
    // per tile shape (BatchShape index)
    CUtensorMap tm_box[kMaxBatchShapes][2];   // halo box of field k
    CUtensorMap tm_tile[kMaxBatchShapes][2];  // tile box of field k
    CUtensorMap tm_v[kMaxBatchShapes];        // tile box of (v dt)^2
    ShotTail<T> s;
};

// Polls of a tile copy's barrier before a block gives up and reports failure.
constexpr unsigned kDefaultWaitLimit = 1u << 24;

template <typename T>
struct BatchConst {
    T az[16], ax[16];  // composed second-derivative coefficients a_0 .. a_l
    T wz[8], wx[8];    // first-derivative weights c_k / d
    float2 az2[16], ax2[16];  // FP32: {a_m, a_m}, operands of the two-cell (packed) instructions
    int nshots;
    int ntiles;  // host bookkeeping only: the kernel ends at the end of its work list
    const int* cta_begin;  // gridDim.x + 1: each CTA's range in `work`
    const int2* work;      // work items (pack_work_item), grouped by CTA
    const int* step_base;  // the launch computes batch step *step_base + step_offset
    int step_offset;
    int* err;              // set when a TMA copy does not arrive in time
    unsigned wait_limit;   // polls of a copy's barrier before the block gives up
    int debug_step;        // test knob (-1: off): at this batch step block 0 withholds its first tile's copies
};

// Device state of a batch of shots sharing the order and the grid spacing.
template <typename T>
class Batch2d {
  public:
    using value_type = T;
    using M = typename MemVar<T>::type;
    Batch2d(int N, double dz, double dx, cudaStream_t stream);

    // Adds a shot: v is the nz x nx model (host or device).  Returns the shot index.  The
    // uploads and the zeroing of its state go to the upload stream (the batch
    // stream unless set_upload_stream was called), where they can overlap
    // batch steps in flight; the caller orders the batch stream after them.
    // On failure the slot is released again.
    int add_shot(const double* v, int64_t nz, int64_t nx, int nB, double dt, int nt, int t_start, bool reverse);
    // Adds a shot on the model of shot k (same grid, bands and dt) with its own
    // state, length and start: the reverse propagation of an RTM shot.
    int add_shot_like(int k, int nt, int t_start, bool reverse);
    // Adds a residual pair (FP32 only): the field P in model vp and the
    // residual D = Q - P of the field Q in model vq (same grid), advanced
    // together so that D keeps FP32 accuracy relative to itself (an RTM
    // shot's dataTrue - dataSmooth is D's row 0).  P's outputs are set on
    // shot(k) as for any shot; D's row 0 goes to shot(k).rec_d.
    int add_pair_shot(const double* vp, const double* vq, int64_t nz, int64_t nx, int nB, double dt, int nt,
                      int t_start);
    ShotTail<T>& shot(int k) { return shots_[k].desc.s; }
    void set_point_sources(int k, int nsrc, const int64_t* iz, const int64_t* ix, const T* d_wavelet);
    void enable(int k, bool on) {
        shots_[k].enabled = on;
        stale_ = true;
    }
    // Releases the device state of shot k; its slot is reused by a later add_shot.
    // The caller must have synchronised the stream past the shot's last step.
    void remove_shot(int k);
    int active_shots() const;
    // Zeroes the fields and memory variables of shot k (upload stream).
    void reset_shot(int k);
    void set_upload_stream(cudaStream_t s) { upload_ = s; }
    // Assigns the tiles of the enabled shots to CTAs (longest-processing-time
    // first, tiles next to a damped band weighted heavier) and uploads every
    // descriptor.  Call again whenever the set of active shots changes.
    void finalize();
    // Re-uploads the descriptor of shot k (after its hooks changed).
    void sync_desc(int k);
    void set_step(int step);
    // Launches `nsteps` batch steps (whole runs of kGraphSteps as graph replays).
    // The schedule must be current: finalize() after any add, remove, enable
    // or point-source change.
    void run(int nsteps);
    // Throws SSSI_ERR_INTERNAL (and clears the flag) when a step's tile copy did
    // not arrive within the wait limit.
    void check_errors();
    // Status of shot k set by the steps (SSSI_OK or SSSI_ERR_UNSTABLE), read
    // after the stream has run; clear_status resets it.
    // the tile shape in use (BatchShape index) and the tuner's last timings
    int tile_shape() const { return shape_; }
    float tuned_ms(int v) const { return tuned_ms_[v]; }
    std::vector<int> statuses();
    void clear_status(int k);
    // Test knob: at batch step `step` block 0 withholds its first tile's copies,
    // and every barrier wait gives up after `wait_limit` polls (step < 0: off,
    // the default limit).
    void set_debug(int step, unsigned wait_limit);
    ~Batch2d();
    Batch2d(const Batch2d&) = delete;
    Batch2d& operator=(const Batch2d&) = delete;
    static constexpr int kGraphSteps = 32;

    const T* current_field(int k) const;  // field after the last completed step of shot k
    int64_t ldp(int k) const { return shots_[k].desc.s.ldp; }
    int L() const { return L_; }
    int grid() const { return grid_; }
    int step_host() const { return step_; }

  private:
    struct Shot {
        ShotDesc<T> desc{};
        bool enabled = true;
        bool free = false;  // slot released by remove_shot
        int64_t origin = 0;
        DeviceBuffer P[2], vdt2, zb, zbm1, zphi[2], zpsi, xb, xbm1, xphi[2], xpsi;
    };
    int N_, L_;
    double dz_, dx_;
    cudaStream_t stream_;
    cudaStream_t upload_ = nullptr;
    bool stale_ = true;  // shots or sources changed since the last finalize
    cudaStream_t up() const { return upload_ ? upload_ : stream_; }
    int take_slot();
    int add_shot_in(int slot, const double* v, int like, int64_t nz, int64_t nx, int nB, double dt, int nt,
                    int t_start, bool reverse, const double* vq = nullptr);
    int pairs_enabled() const;
    void ensure_status();
    BatchConst<T> bc_{};
    std::vector<Shot> shots_;
    void launch_step(const int* base, int offset, cudaStream_t stream);
    void drop_graph();
    // launch parameters the graph was captured with (the work list and the
    // descriptors are read from device memory, so only these invalidate it)
    struct GraphKey {
        int grid = 0;
        bool split = false;
        bool pair = false;
        bool lean = false;
        int shape = 0;
        const void *desc = nullptr, *begin = nullptr, *work = nullptr;
        int debug_step = -1;
        unsigned wait_limit = 0;
        bool operator==(const GraphKey& o) const {
            return grid == o.grid && split == o.split && pair == o.pair && lean == o.lean && shape == o.shape && desc == o.desc &&
                   begin == o.begin && work == o.work && debug_step == o.debug_step && wait_limit == o.wait_limit;
        }
    } graph_key_;
    GraphKey current_key() const {
        return GraphKey{grid_, split_, pair_, lean_, shape_, d_desc_.get(), d_cta_begin_[shape_].get(),
                        d_work_[shape_].get(), bc_.debug_step, bc_.wait_limit};
    }
    // tile shape: the schedule in use (BatchShape index) and the tuner (times a
    // few steps with each shape when a large schedule is built, keeps the faster)
    int shape_ = 0;
    bool tune_ = false;
    int tuned_tiles_ = 0;
    float tuned_ms_[kMaxBatchShapes] = {};  // the tuner's last timing of each shape
    static constexpr int kTuneSteps = 6, kTuneMinRun = 64;  // steps per shape; shortest run that tunes
    int tile_z(int shape) const;
    int tile_x(int shape) const;
    void schedule(int shape);  // work lists of the enabled shots for a tile shape
    void use_shape(int shape);
    bool split_ = false;  // the schedule holds half tiles
    bool pair_ = false;   // enabled residual pairs: the launch uses the pair variant (32 x 32 tiles)
    bool lean_ = false;   // no enabled shot has rare outputs: the variant without them
    void update_lean();   // from the descriptors as uploaded
    int shape_free_ = 0;  // the tile shape to return to when the last pair leaves
    DeviceBuffer d_desc_, d_ctr_;                // d_ctr_: graph step base, zero, error flag
    DeviceBuffer d_status_;                      // one status word per shot slot
    DeviceBuffer d_cta_begin_[kMaxBatchShapes], d_work_[kMaxBatchShapes];  // the schedule of each tile shape
    int grid_s_[kMaxBatchShapes] = {}, ntiles_s_[kMaxBatchShapes] = {};
    bool split_s_[kMaxBatchShapes] = {};
    int grid_ = 0, ntiles_ = 0, step_ = 0;
    int ctas_per_sm_[kMaxBatchShapes] = {1, 1, 1}, ctas_per_sm_pair_ = 1, sms_ = 1;
    cudaGraphExec_t graph_ = nullptr;
};

// Launches one batch step with the programmatic-serialization attribute.
// split: the work lists hold half tiles; shape: BatchShape index; pair: the
// batch holds residual pairs (FP32, shape 1, no half tiles); lean: no shot
// writes snapshots, FP16 packs, maxima or imaging sums (the variant without
// those outputs; whole tiles only).
template <typename T, int N>
void launch_batch2d_n(const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, bool split, int shape, bool pair,
                      bool lean, cudaStream_t stream);
template <typename T, int N>
int batch2d_occupancy_n(int shape, bool pair);
template <typename T>
void launch_batch2d(int N, const ShotDesc<T>* shots, const BatchConst<T>& bc, int grid, bool split, int shape,
                    bool pair, bool lean, cudaStream_t stream);
template <typename T>
int batch2d_ctas_per_sm(int N, int shape, bool pair);

}  // namespace sssi
