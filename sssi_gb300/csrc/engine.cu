// Plans: many shots resident on one GPU, advanced together (continuous
// batching), admitted by device-memory footprint.  See the plan API in
// sssi_gb300.h.
//
// One worker thread per plan owns a CUDA stream and all device state:
//   - 2D shots (forward modelling, RTM) live in one Batch2d: every launch of
//     the batched step advances all of them by one step.  A shot joins at the
//     batch step at which it is admitted (its t_start) and is removed when its
//     last step has run, so the tiles of finished shots leave the schedule
//     and their memory returns to the pool.
//   - An RTM request is three batch shots, as in the single-shot RTM: forward
//     in v and in vs over its first nt steps, reverse in v over the next nt
//     (added at admission, enabled at the phase change, when the FP16 pack of
//     the last forward step and dataTrue - dataSmooth are computed).
//   - 3D shots each keep a Prop3d and advance by up to steps_per_round steps
//     per round.
// Rounds end at the next event of any 2D shot (a phase change or a shot's
// end), so events always fall on round boundaries.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <thread>

#include "api_util.cuh"
#include "batch2d.cuh"
#include "cpml2d.cuh"
#include "prop3d.cuh"

namespace sssi {

namespace {

using namespace api;
using Clock = std::chrono::steady_clock;

// FP16 snapshot scale blocks (32 x 32 cells) of an nz x nx grid.
inline int64_t nblocks(int64_t nz, int64_t nx) { return ((nz + 31) / 32) * ((nx + 31) / 32); }

// Device array of T -> caller array of doubles (host or device).
template <typename T>
void deliver(const T* dev, size_t n, double* out, cudaStream_t s) {
    if (!out || n == 0) return;
    const bool out_dev = is_device_pointer(out);
    if (std::is_same<T, double>::value) {
        SSSI_CHECK_CUDA(cudaMemcpyAsync(out, dev, n * sizeof(double),
                                        out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    } else if (out_dev) {
        convert(dev, out, (int64_t)n, s);
    } else {
        DeviceBuffer tmp(n * sizeof(double));
        convert(dev, tmp.as<double>(), (int64_t)n, s);
        SSSI_CHECK_CUDA(cudaMemcpyAsync(out, tmp.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s));  // before tmp returns to the pool
    }
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

// stack[i + j * ld] += img[i + j * nz]: one shot's image into a plan's stack.
__global__ void stack_add_kernel(const double* img, int64_t nz, int64_t nx, double* stack, int64_t ld) {
    const int64_t n = nz * nx;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        stack[(q % nz) + (q / nz) * ld] += img[q];
}

// Host doubles -> new device array of T.
template <typename T>
void upload(DeviceBuffer& buf, const std::vector<double>& h, cudaStream_t s) {
    buf.allocate(sizeof(T) * std::max<size_t>(h.size(), 1));
    if (h.empty()) return;
    std::vector<T> t(h.begin(), h.end());
    SSSI_CHECK_CUDA(cudaMemcpyAsync(buf.get(), t.data(), sizeof(T) * t.size(), cudaMemcpyHostToDevice, s));
    SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

struct PlanRequest {
    int64_t ticket = 0;
    sssi_shot_desc d{};
    std::vector<double> v, vs, wav;
    std::vector<int64_t> iz, ix, iy;
    int state = SSSI_SHOT_QUEUED;
    int status = SSSI_OK;
    std::string msg;
    double t_submit = 0, t_start = 0, t_done = 0;
    size_t bytes = 0;
    int64_t cells = 0;
    std::atomic<bool> cancel{false};  // set by sssi_cancel; the worker drops the shot at its next round
    double* stack_ptr = nullptr;      // RTM: the stack window the image is added to (ld = stack_ld)
    int64_t stack_ld = 0;
};
using ReqPtr = std::shared_ptr<PlanRequest>;

// The outputs of a finished shot, copied out by the plan's delivery thread on
// its own stream (after `ready`, recorded on the batch stream once the shot's
// last work is queued), so the batch keeps stepping meanwhile.
struct Delivery {
    ReqPtr r;
    cudaEvent_t ready = nullptr;
    std::function<void(cudaStream_t)> copy;
    std::shared_ptr<void> keep;  // device buffers the copy reads
};

class EngineBase {
  public:
    virtual ~EngineBase() = default;
    virtual size_t footprint(const PlanRequest& r) const = 0;
    virtual void admit(const ReqPtr& r) = 0;
    // A round in two halves, so that admitting new shots (host work and
    // uploads on a side stream) overlaps the steps in flight:
    // launch() queues the next steps of every admitted shot and returns the
    // cell-updates queued; complete() waits for them, checks the kernels'
    // error flags and handles the shots' events.  Finished shots are appended
    // to `out` (their outputs still to be copied).
    virtual double launch(std::vector<Delivery>& out) = 0;
    virtual void complete(std::vector<Delivery>& out) = 0;
    virtual bool busy() const = 0;
    virtual void fail_all(std::vector<ReqPtr>& fin, const std::string& why) = 0;
    // Shots that failed on their own (a blow-up) or were cancelled since the
    // last call; the others keep running.
    void take_failed(std::vector<ReqPtr>& fin) {
        fin.insert(fin.end(), failed_.begin(), failed_.end());
        failed_.clear();
    }
    virtual int64_t batch_steps() const = 0;
    std::vector<ReqPtr> failed_;
    double gpu_wait_s = 0;  // host time blocked on the batch stream
    // device time of the batched 2D steps (CUDA events around each round's
    // launches) and the cell-updates they made
    double batch2d_gpu_s = 0, batch2d_cells = 0;
    // the batched step's tile shape in use and the tuner's timings of each
    int tile_shape = 0;
    double tune_ms[3] = {0, 0, 0};

  protected:
    // Waits for the batch stream, counting the time.
    void wait_stream(cudaStream_t s) {
        const auto t = Clock::now();
        const cudaError_t e = cudaStreamSynchronize(s);
        gpu_wait_s += std::chrono::duration<double>(Clock::now() - t).count();
        SSSI_CHECK_CUDA(e);
    }
};

template <typename T>
class Engine final : public EngineBase {
    using M = typename MemVar<T>::type;
    static constexpr bool kF16 = std::is_same<T, float>::value;

    struct Run {
        ReqPtr r;
        int kA = -1, kB = -1, kR = -1;
        int64_t s0 = 0;
        int phase = 1;
        DeviceBuffer wav, recA, recB, delta, fsnap, amax, perr, Mb, S2, img;
        std::unique_ptr<Prop3d<T>> p3;
        int64_t done3 = 0;
        cudaStream_t s3 = nullptr;  // 3D: the propagation's own stream (runs beside the 2D batch)
        ~Run() {
            p3.reset();
            if (s3) cudaStreamDestroy(s3);  // released once its work has completed
        }
    };

  public:
    Engine(const sssi_plan_config& c, cudaStream_t s)
        : cfg_(c), s_(s), B_(c.nDiffOrder, c.dz, c.dx, s), rounds_(c.steps_per_round > 0 ? c.steps_per_round : 64) {
        SSSI_CHECK_CUDA(cudaStreamCreateWithFlags(&up_, cudaStreamNonBlocking));
        SSSI_CHECK_CUDA(cudaEventCreateWithFlags(&up_done_, cudaEventDisableTiming));
        SSSI_CHECK_CUDA(cudaEventCreate(&ev2_[0]));
        SSSI_CHECK_CUDA(cudaEventCreate(&ev2_[1]));
        B_.set_upload_stream(up_);
    }
    ~Engine() override {
        cudaStreamSynchronize(up_);
        cudaEventDestroy(up_done_);
        cudaEventDestroy(ev2_[0]);
        cudaEventDestroy(ev2_[1]);
        cudaStreamDestroy(up_);
    }

    size_t footprint(const PlanRequest& r) const override {
        const int N = cfg_.nDiffOrder, L = 2 * N - 1, HZ = tile_halo_rows(N);
        const size_t ts = sizeof(T), ms = sizeof(M);
        const int64_t nz = r.d.nz, nx = r.d.nx, ny = r.d.ny, nt = r.d.nt, nB = r.d.nBoundary;
        auto shot2d = [&]() -> size_t {
            const int64_t ldp = nz + 2 * std::max(L, HZ) + 2 * TileShape<T>::TZ;
            const size_t field = ts * (size_t)ldp * (size_t)(nx + 2 * L);
            const size_t band = (size_t)(nB * nx + nz * 2 * nB);
            return 3 * field + band * (2 * ts + 3 * ms);
        };
        const size_t wav = ts * (size_t)(std::max(r.d.nsrc, 1) * std::max<int64_t>(nt, 1));
        if (r.d.kind == SSSI_SHOT_FWD2D) return shot2d() + ts * (size_t)(nx * nt) + wav;
        if (r.d.kind == SSSI_SHOT_RTM2D) {
            const size_t n = (size_t)(nz * nx);
            const int stride = kF16 ? (r.d.snap_stride > 0 ? r.d.snap_stride : 4) : 1;
            const size_t nsnap = (size_t)((nt + stride - 1) / stride);
            const size_t snaps = kF16 ? 2 * n * nsnap + 4 * (size_t)nblocks(nz, nx) * nsnap + 4 * n : 8 * n * (size_t)nt;
            return 3 * shot2d() + 3 * ts * (size_t)(nx * nt) + snaps + 16 * n + wav;
        }
        const int64_t vol = (nz + 2 * HZ + 3) * (nx + 2 * L) * (ny + 2 * L);
        const size_t band3 = (size_t)(nB * nx * ny + nz * 2 * nB * ny + nz * nx * 2 * nB);
        const size_t ms3 = sizeof(typename MemVar3<T>::type);
        return 3 * ts * (size_t)vol + 3 * ms3 * band3 + ts * (size_t)(nx * ny * nt) + wav + 8 * (size_t)(nz * nx * ny);
    }

    void admit(const ReqPtr& r) override {
        auto u = std::make_unique<Run>();
        u->r = r;
        const sssi_shot_desc& d = r->d;
        const int64_t nz = d.nz, nx = d.nx, nt = d.nt;
        upload<T>(u->wav, r->wav, up_);
        if (d.kind == SSSI_SHOT_FWD3D) {
            // set up on the upload stream, stepped on the batch stream
            u->p3 = std::make_unique<Prop3d<T>>(r->v.data(), nz, nx, d.ny, cfg_.nDiffOrder, d.nBoundary, cfg_.dz,
                                                cfg_.dx, cfg_.dy, d.dt, (int)nt, up_);
            if (d.nsrc)
                u->p3->set_point_sources(d.nsrc, r->iz.data(), r->ix.data(), r->iy.data(), u->wav.template as<T>());
            u->recA.allocate(sizeof(T) * std::max<int64_t>(nx * d.ny * nt, 1));
            u->p3->desc().rec = u->recA.template as<T>();
            u->p3->sync_desc();
            SSSI_CHECK_CUDA(cudaStreamCreateWithFlags(&u->s3, cudaStreamNonBlocking));
            u->p3->set_stream(u->s3);
            SSSI_CHECK_CUDA(cudaEventRecord(up_done_, up_));
            r->cells = nz * nx * d.ny * nt;
            runs3_.push_back(std::move(u));
            return;
        }
        try {
            admit2d(*u);
        } catch (...) {
            const int ks[3] = {u->kA, u->kB, u->kR};
            for (int k : ks)
                if (k >= 0) B_.remove_shot(k);
            throw;
        }
        SSSI_CHECK_CUDA(cudaEventRecord(up_done_, up_));
        dirty_ = true;
        runs2_.push_back(std::move(u));
    }

  private:
    void admit2d(Run& ru) {
        Run* u = &ru;
        const ReqPtr& r = u->r;
        const sssi_shot_desc& d = r->d;
        const int64_t nz = d.nz, nx = d.nx, nt = d.nt;
        u->s0 = step_;
        const size_t ndata = (size_t)(nx * std::max<int64_t>(nt, 1));
        if (d.kind == SSSI_SHOT_FWD2D) {
            u->kA = B_.add_shot(r->v.data(), nz, nx, d.nBoundary, d.dt, (int)nt, (int)step_, false);
            B_.set_point_sources(u->kA, d.nsrc, r->iz.data(), r->ix.data(), u->wav.template as<T>());
            u->recA.allocate(sizeof(T) * ndata);
            B_.shot(u->kA).rec = u->recA.template as<T>();
            r->cells = nz * nx * nt;
        } else {
            const int64_t n = nz * nx;
            const int stride = kF16 ? (d.snap_stride > 0 ? d.snap_stride : 4) : 1;
            const int64_t nsnap = (nt + stride - 1) / stride;
            // FP32: the field in vs and the residual (field in v) - (field in vs)
            // as one residual pair (dataTrue - dataSmooth is the residual's row
            // 0, accurate relative to itself); FP64: two forward shots
            if (kF16) {
                u->kB = B_.add_pair_shot(r->vs.data(), r->v.data(), nz, nx, d.nBoundary, d.dt, (int)nt, (int)step_);
                u->kR = B_.add_shot(r->v.data(), nz, nx, d.nBoundary, d.dt, (int)nt, (int)(step_ + nt), true);
            } else {
                u->kA = B_.add_shot(r->v.data(), nz, nx, d.nBoundary, d.dt, (int)nt, (int)step_, false);
                u->kB = B_.add_shot(r->vs.data(), nz, nx, d.nBoundary, d.dt, (int)nt, (int)step_, false);
                u->kR = B_.add_shot_like(u->kA, (int)nt, (int)(step_ + nt), true);
                B_.set_point_sources(u->kA, 1, r->iz.data(), r->ix.data(), u->wav.template as<T>());
            }
            B_.enable(u->kR, false);
            B_.set_point_sources(u->kB, 1, r->iz.data(), r->ix.data(), u->wav.template as<T>());
            u->recA.allocate(sizeof(T) * ndata);
            u->recB.allocate(sizeof(T) * ndata);
            u->delta.allocate(sizeof(T) * ndata);
            u->Mb.allocate(sizeof(double) * n);
            u->S2.allocate(sizeof(double) * n);
            u->Mb.zero(up_);
            if (kF16) {
                u->fsnap.allocate(sizeof(__half) * n * std::max<int64_t>(nsnap, 1));
                u->amax.allocate(sizeof(unsigned) * nblocks(nz, nx) * std::max<int64_t>(nsnap, 1));
                u->amax.zero(up_);
                u->perr.allocate(sizeof(float) * n);
                u->perr.zero(up_);
                u->S2.zero(up_);
            } else {
                u->fsnap.allocate(sizeof(double) * n * std::max<int64_t>(nt, 1));
                fill(u->S2.template as<double>(), n, d.epsilon, up_);
            }
            if (u->kA >= 0) B_.shot(u->kA).rec = u->recA.template as<T>();
            ShotTail<T>& b = B_.shot(u->kB);
            b.rec = u->recB.template as<T>();
            if (kF16) b.rec_d = u->delta.template as<T>();
            if (kF16) {
                b.stride = stride;
                b.amax = u->amax.template as<unsigned>();
                b.pack = u->fsnap.template as<__half>();
                b.s2acc = u->S2.template as<float2>();  // the illumination from the FP32 forward field
                b.perr = u->perr.template as<float>();
            } else {
                b.snap = reinterpret_cast<T*>(u->fsnap.template as<double>());
                b.snap_t0 = 0;
            }
            ShotTail<T>& rr = B_.shot(u->kR);
            rr.src_row = u->delta.template as<T>();
            if (kF16) {
                rr.stride = stride;
                rr.img_f16 = u->fsnap.template as<__half>();
                rr.img_amax = u->amax.template as<unsigned>();
                rr.img_m2 = u->Mb.template as<float2>();
            } else {
                rr.img_f64 = u->fsnap.template as<double>();
                rr.img_m = u->Mb.template as<double>();
                rr.img_s2 = u->S2.template as<double>();
            }
            r->cells = 3 * n * nt;
        }
    }

  public:
    bool busy() const override { return !runs2_.empty() || !runs3_.empty(); }
    int64_t batch_steps() const override { return launches_; }

    double launch(std::vector<Delivery>& out) override {
        double cells = 0;
        ran2_ = false;
        drop_cancelled();  // every stream is idle here: the last round has completed
        finish_2d_events(out);  // zero-step shots and events due right at admission
        SSSI_CHECK_CUDA(cudaStreamWaitEvent(s_, up_done_, 0));  // uploads of the shots admitted so far
        // ---- 2D batch: up to the next event of any shot
        if (!runs2_.empty()) {
            int64_t K = rounds_;
            for (auto& u : runs2_) K = std::min(K, next_event(*u) - step_);
            K = std::max<int64_t>(K, 1);
            if (dirty_) {
                B_.finalize();
                dirty_ = false;
            }
            B_.set_step((int)step_);
            SSSI_CHECK_CUDA(cudaEventRecord(ev2_[0], s_));
            B_.run((int)K);
            SSSI_CHECK_CUDA(cudaEventRecord(ev2_[1], s_));
            cells2_ = 0;
            for (auto& u : runs2_) {
                const int64_t n = (int64_t)u->r->d.nz * u->r->d.nx;
                cells2_ += (double)n * K * (u->r->d.kind == SSSI_SHOT_RTM2D && u->phase == 1 ? 2 : 1);
            }
            cells += cells2_;
            step_ += K;
            launches_ += K;
            ran2_ = true;
        }
        // ---- 3D shots: up to steps_per_round steps each, each on its own stream
        // (the persistent kernels of the batch and of the 3D shots fill one
        // another's idle SMs)
        for (auto& up : runs3_) {
            Run& u = *up;
            const int64_t k = std::min<int64_t>(rounds_, u.r->d.nt - u.done3);
            if (k > 0) {
                SSSI_CHECK_CUDA(cudaStreamWaitEvent(u.s3, up_done_, 0));
                u.p3->run((int)k);
                u.done3 += k;
                cells += (double)u.r->d.nz * u.r->d.nx * u.r->d.ny * k;
            }
        }
        return cells;
    }

    void complete(std::vector<Delivery>& out) override {
        wait_stream(s_);
        for (auto& up : runs3_) wait_stream(up->s3);
        if (ran2_) {
            float ms = 0;
            SSSI_CHECK_CUDA(cudaEventElapsedTime(&ms, ev2_[0], ev2_[1]));
            batch2d_gpu_s += 1e-3 * ms;
            batch2d_cells += cells2_;
            tile_shape = B_.tile_shape();
            for (int v = 0; v < 3; ++v) tune_ms[v] = v < kBatchShapes<T> ? B_.tuned_ms(v) : 0.0f;
            B_.check_errors();
            fail_unstable();
            finish_2d_events(out);
        }
        ran2_ = false;
        for (size_t q = 0; q < runs3_.size();) {
            Run& u = *runs3_[q];
            const int64_t nt = u.r->d.nt;
            if (u.done3 >= nt) {
                u.p3->check_errors();
                const T* rec = u.recA.template as<T>();
                const size_t n = (size_t)(u.r->d.nx * u.r->d.ny * nt);
                double* dst = u.r->d.data;
                cudaStream_t s3 = u.s3;
                hand_over(std::move(runs3_[q]), out, [=](cudaStream_t cs) { deliver<T>(rec, n, dst, cs); }, s3);
                runs3_.erase(runs3_.begin() + q);
                continue;
            }
            ++q;
        }
    }

    void fail_all(std::vector<ReqPtr>& fin, const std::string& why) override {
        cudaStreamSynchronize(s_);
        cudaStreamSynchronize(up_);
        for (auto& u : runs3_)
            if (u->s3) cudaStreamSynchronize(u->s3);
        ran2_ = false;
        for (auto& u : runs2_) {
            u->r->status = SSSI_ERR_INTERNAL;
            u->r->msg = why;
            fin.push_back(u->r);
            const int ks[3] = {u->kA, u->kB, u->kR};
            for (int k : ks)
                if (k >= 0) B_.remove_shot(k);
        }
        for (auto& u : runs3_) {
            u->r->status = SSSI_ERR_INTERNAL;
            u->r->msg = why;
            fin.push_back(u->r);
        }
        runs2_.clear();
        runs3_.clear();
        dirty_ = true;
    }

  private:
    // Removes run q of runs2_ (its shots leave the batch) and reports it failed.
    void fail_run2(size_t q, int status, const std::string& why) {
        Run& u = *runs2_[q];
        const int ks[3] = {u.kA, u.kB, u.kR};
        for (int k : ks)
            if (k >= 0) B_.remove_shot(k);
        u.r->status = status;
        u.r->msg = why;
        failed_.push_back(u.r);
        runs2_.erase(runs2_.begin() + q);
        dirty_ = true;
    }

    // A shot whose receiver row went non-finite fails alone; the batch goes on.
    void fail_unstable() {
        const std::vector<int> st = B_.statuses();
        auto bad = [&](int k) { return k >= 0 && k < (int)st.size() && st[k] == SSSI_ERR_UNSTABLE; };
        for (size_t q = 0; q < runs2_.size();) {
            const Run& u = *runs2_[q];
            if (bad(u.kA) || bad(u.kB) || bad(u.kR))
                fail_run2(q, SSSI_ERR_UNSTABLE,
                          "the wavefield became non-finite (is dt beyond the stability limit of the grid and the "
                          "velocities?)");
            else
                ++q;
        }
    }

    // Cancelled shots leave at a round boundary, when none of their work is in flight.
    void drop_cancelled() {
        for (size_t q = 0; q < runs2_.size();) {
            if (runs2_[q]->r->cancel.load())
                fail_run2(q, SSSI_ERR_CANCELLED, "cancelled");
            else
                ++q;
        }
        for (size_t q = 0; q < runs3_.size();) {
            if (runs3_[q]->r->cancel.load()) {
                runs3_[q]->r->status = SSSI_ERR_CANCELLED;
                runs3_[q]->r->msg = "cancelled";
                failed_.push_back(runs3_[q]->r);
                runs3_.erase(runs3_.begin() + q);
            } else {
                ++q;
            }
        }
    }

    int64_t next_event(const Run& u) const {
        const int64_t nt = u.r->d.nt;
        if (u.r->d.kind == SSSI_SHOT_RTM2D) return u.s0 + (u.phase == 1 ? nt : 2 * nt);
        return u.s0 + nt;
    }

    // Queues the delivery of a finished run's outputs; the run (and its device
    // buffers) lives until the copies are done.
    template <class F>
    void hand_over(std::unique_ptr<Run> u, std::vector<Delivery>& out, F&& copy, cudaStream_t s = nullptr) {
        Delivery dl;
        dl.r = u->r;
        SSSI_CHECK_CUDA(cudaEventCreateWithFlags(&dl.ready, cudaEventDisableTiming));
        SSSI_CHECK_CUDA(cudaEventRecord(dl.ready, s ? s : s_));
        dl.copy = std::forward<F>(copy);
        dl.keep = std::shared_ptr<Run>(std::move(u));
        out.push_back(std::move(dl));
    }

    void finish_2d_events(std::vector<Delivery>& out) {
        for (size_t q = 0; q < runs2_.size();) {
            Run& u = *runs2_[q];
            if (step_ < next_event(u)) {
                ++q;
                continue;
            }
            const sssi_shot_desc& d = u.r->d;
            const int64_t nz = d.nz, nx = d.nx, nt = d.nt, n = nz * nx;
            if (d.kind == SSSI_SHOT_FWD2D) {
                B_.remove_shot(u.kA);
                const T* rec = u.recA.template as<T>();
                double* dst = d.data;
                const size_t cnt = (size_t)(nx * nt);
                hand_over(std::move(runs2_[q]), out, [=](cudaStream_t cs) { deliver<T>(rec, cnt, dst, cs); });
                runs2_.erase(runs2_.begin() + q);
                dirty_ = true;
                continue;
            } else if (u.phase == 1) {
                // forward phase done: FP16 pack of the last forward step, residual data
                const int stride = kF16 ? (d.snap_stride > 0 ? d.snap_stride : 4) : 1;
                if (kF16 && nt >= 1 && (nt - 1) % stride == 0) {
                    const int64_t k = (nt - 1) / stride;
                    launch_pack_f16(reinterpret_cast<const float*>(B_.current_field(u.kB)), B_.ldp(u.kB), (int)nz,
                                    (int)nx, u.amax.template as<unsigned>() + k * nblocks(nz, nx),
                                    u.fsnap.template as<__half>() + k * n, u.perr.template as<float>(), s_);
                }
                if (nt > 0) {
                    // the reverse source dataTrue - dataSmooth: the residual's row 0
                    // (FP32), or the difference of the two forward shots (FP64);
                    // dataTrue itself (FP32) as dataSmooth + residual, when wanted
                    if (!kF16)
                        diff_kernel<T><<<152 * 4, 256, 0, s_>>>(u.recA.template as<T>(), u.recB.template as<T>(),
                                                                u.delta.template as<T>(), nx * nt);
                    else if (d.data)
                        sum_kernel<T><<<152 * 4, 256, 0, s_>>>(u.recB.template as<T>(), u.delta.template as<T>(),
                                                               u.recA.template as<T>(), nx * nt);
                    if (!kF16 || d.data) count_launch();
                    SSSI_CHECK_CUDA(cudaGetLastError());
                }
                wait_stream(s_);
                if (u.kA >= 0) B_.remove_shot(u.kA);
                B_.remove_shot(u.kB);
                u.kA = u.kB = -1;
                B_.enable(u.kR, true);
                u.phase = 2;
                dirty_ = true;
                ++q;  // its reverse phase ends nt steps later
                continue;
            } else {
                u.img.allocate(sizeof(double) * std::max<int64_t>(n, 1));
                const int stride = kF16 ? (d.snap_stride > 0 ? d.snap_stride : 4) : 1;
                if (kF16)
                    image_finish_comp_kernel<<<152 * 4, 256, 0, s_>>>(u.Mb.template as<float2>(),
                                                                       u.S2.template as<float2>(), n, (double)stride,
                                                                       d.epsilon, u.img.template as<double>());
                else
                    image_finish_kernel<<<152 * 4, 256, 0, s_>>>(u.Mb.template as<double>(), u.S2.template as<double>(),
                                                                  n, 1.0, 0.0, u.img.template as<double>());
                count_launch();
                SSSI_CHECK_CUDA(cudaGetLastError());
                if (u.r->stack_ptr) {  // ordered before the delivery's event: done means added
                    stack_add_kernel<<<152 * 4, 256, 0, s_>>>(u.img.template as<double>(), nz, nx, u.r->stack_ptr,
                                                              u.r->stack_ld);
                    count_launch();
                    SSSI_CHECK_CUDA(cudaGetLastError());
                }
                B_.remove_shot(u.kR);
                const double* img = u.img.template as<double>();
                const T* rec = u.recA.template as<T>();
                double *dimg = d.image, *ddata = d.data;
                const size_t cimg = (size_t)n, cdata = (size_t)(nx * nt);
                hand_over(std::move(runs2_[q]), out, [=](cudaStream_t cs) {
                    deliver<double>(img, cimg, dimg, cs);
                    if (ddata) deliver<T>(rec, cdata, ddata, cs);
                });
                runs2_.erase(runs2_.begin() + q);
                dirty_ = true;
            }
        }
    }

    sssi_plan_config cfg_;
    cudaStream_t s_;
    cudaStream_t up_ = nullptr;     // admission: uploads and zeroing of new shots
    cudaEvent_t up_done_ = nullptr; // recorded after each admission; the batch stream waits on it
    bool ran2_ = false;             // the round in flight has 2D steps
    cudaEvent_t ev2_[2] = {nullptr, nullptr};  // around the 2D launches of the round in flight
    double cells2_ = 0;                        // their cell-updates
    Batch2d<T> B_;
    int64_t rounds_;
    int64_t step_ = 0, launches_ = 0;
    bool dirty_ = true;
    std::vector<std::unique_ptr<Run>> runs2_, runs3_;
};

}  // namespace sssi

struct sssi_plan {
    sssi_plan_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    sssi::Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<sssi::ReqPtr> queue;
    std::map<int64_t, sssi::ReqPtr> tickets;
    int64_t next_ticket = 1;
    size_t budget = 0, in_use = 0;
    int64_t n_running = 0, n_done = 0, n_failed = 0, batch_steps = 0;
    double cells = 0, admit_s = 0, round_s = 0, gpu_wait_s = 0, deliver_s = 0, batch2d_gpu_s = 0,
           batch2d_cells = 0;
    int tile_shape = 0;
    double tune_ms[3] = {0, 0, 0};
    bool stop = false;
    int fatal = SSSI_OK;
    std::string fatal_msg;
    std::unique_ptr<sssi::EngineBase> engine;
    std::thread worker;
    // stacked images (sssi_plan_stack_create): device memory and the shots still to add
    struct Stack {
        sssi::DeviceBuffer buf;
        int64_t nz = 0, nx = 0, pending = 0;
    };
    std::map<int64_t, std::unique_ptr<Stack>> stacks;
    int64_t next_stack = 1;
    // delivery thread: copies finished shots' outputs on its own stream
    cudaStream_t dstream = nullptr;
    std::deque<sssi::Delivery> deliveries;
    std::condition_variable cv_deliver;
    bool deliver_stop = false;
    std::thread deliverer;

    double now() const { return std::chrono::duration<double>(sssi::Clock::now() - t0).count(); }

    void finish(std::vector<sssi::ReqPtr>& fin) {
        std::lock_guard<std::mutex> lk(mu);
        for (auto& r : fin) {
            if (r->d.stack) {
                auto it = stacks.find(r->d.stack);
                if (it != stacks.end()) --it->second->pending;
            }
            r->t_done = now();
            r->state = r->status == SSSI_OK ? SSSI_SHOT_DONE : SSSI_SHOT_FAILED;
            in_use -= std::min(in_use, r->bytes);
            --n_running;
            (r->status == SSSI_OK ? n_done : n_failed) += 1;
        }
        fin.clear();
        cv_done.notify_all();
        cv_work.notify_all();  // memory came back: a queued shot may fit now
    }

    // The next queued shot fits the memory not held by admitted or delivering
    // shots (a shot larger than the whole budget runs alone).
    bool front_fits() const {
        return !queue.empty() && (in_use == 0 || in_use + queue.front()->bytes <= budget);
    }

    void hand_over(std::vector<sssi::Delivery>& out) {
        if (out.empty()) return;
        {
            std::lock_guard<std::mutex> lk(mu);
            for (auto& d : out) deliveries.push_back(std::move(d));
        }
        out.clear();
        cv_deliver.notify_one();
    }

    void deliver_loop() {
        cudaSetDevice(device);
        std::vector<sssi::ReqPtr> fin;
        while (true) {
            sssi::Delivery d;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_deliver.wait(lk, [&] { return deliver_stop || !deliveries.empty(); });
                if (deliveries.empty()) break;  // stopped and drained
                d = std::move(deliveries.front());
                deliveries.pop_front();
            }
            sssi::clear_error();
            const auto td = sssi::Clock::now();
            try {
                SSSI_CHECK_CUDA(cudaStreamWaitEvent(dstream, d.ready, 0));
                d.copy(dstream);
                SSSI_CHECK_CUDA(cudaStreamSynchronize(dstream));
            } catch (const sssi::Error& e) {
                d.r->status = e.code;
                d.r->msg = std::string("output copy failed: ") + sssi_last_error();
            } catch (...) {
                d.r->status = SSSI_ERR_INTERNAL;
                d.r->msg = "output copy failed: unexpected exception";
            }
            cudaStreamSynchronize(dstream);
            cudaEventDestroy(d.ready);
            d.keep.reset();
            {
                std::lock_guard<std::mutex> lk(mu);
                deliver_s += std::chrono::duration<double>(sssi::Clock::now() - td).count();
            }
            fin.push_back(d.r);
            finish(fin);
        }
    }

    // Admits the queued shots that fit, first come first served.
    void admit_queued(std::vector<sssi::ReqPtr>& fin) {
        std::vector<sssi::ReqPtr> admit;
        {
            std::lock_guard<std::mutex> lk(mu);
            while (front_fits()) {
                sssi::ReqPtr& r = queue.front();
                in_use += r->bytes;
                r->state = SSSI_SHOT_RUNNING;
                r->t_start = now();
                ++n_running;
                admit.push_back(r);
                queue.pop_front();
            }
        }
        if (admit.empty()) return;
        const auto ta = sssi::Clock::now();
        for (auto& r : admit) {
            sssi::clear_error();
            try {
                engine->admit(r);
            } catch (const sssi::Error& e) {
                r->status = e.code;
                r->msg = sssi_last_error();
                fin.push_back(r);
            } catch (const std::bad_alloc&) {
                r->status = SSSI_ERR_NOMEM;
                r->msg = "host allocation failed";
                fin.push_back(r);
            } catch (...) {
                r->status = SSSI_ERR_INTERNAL;
                r->msg = "unexpected exception while admitting the shot";
                fin.push_back(r);
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        admit_s += std::chrono::duration<double>(sssi::Clock::now() - ta).count();
    }

    // Runs one half of a round; a failure fails every admitted shot (they
    // share the batch and its stream).
    template <class F>
    bool guarded_step(std::vector<sssi::ReqPtr>& fin, F&& f) {
        try {
            f();
            return true;
        } catch (const sssi::Error&) {
            engine->fail_all(fin, std::string("batch step failed: ") + sssi_last_error());
        } catch (...) {
            engine->fail_all(fin, "batch step failed: unexpected exception");
        }
        return false;
    }

    void run() {
        cudaSetDevice(device);
        std::vector<sssi::ReqPtr> fin;
        std::vector<sssi::Delivery> out;
        while (true) {
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return stop || front_fits() || engine->busy(); });
                if (stop) break;
            }
            const auto t0r = sssi::Clock::now();
            const double admit0 = admit_s;
            double c = 0;
            bool ok = guarded_step(fin, [&] { c = engine->launch(out); });
            admit_queued(fin);  // overlaps the steps just launched
            if (ok) ok = guarded_step(fin, [&] { engine->complete(out); });
            engine->take_failed(fin);
            {
                std::lock_guard<std::mutex> lk(mu);
                if (ok) cells += c;
                batch_steps = engine->batch_steps();
                round_s += std::chrono::duration<double>(sssi::Clock::now() - t0r).count() - (admit_s - admit0);
                gpu_wait_s = engine->gpu_wait_s;
                batch2d_gpu_s = engine->batch2d_gpu_s;
                batch2d_cells = engine->batch2d_cells;
                tile_shape = engine->tile_shape;
                for (int v = 0; v < 3; ++v) tune_ms[v] = engine->tune_ms[v];
            }
            hand_over(out);
            if (!fin.empty()) finish(fin);
        }
        // plan destroyed: fail what is left
        engine->fail_all(fin, "plan destroyed");
        {
            std::lock_guard<std::mutex> lk(mu);
            for (auto& r : queue) {
                r->status = SSSI_ERR_INTERNAL;
                r->msg = "plan destroyed";
                r->state = SSSI_SHOT_FAILED;
                ++n_failed;
            }
            queue.clear();
        }
        finish(fin);
        engine.reset();
        cudaStreamSynchronize(stream);
    }
};

namespace {

using namespace sssi;

void fill_info(const PlanRequest& r, sssi_shot_info* info) {
    if (!info) return;
    info->state = r.state;
    info->status = r.status;
    info->submit_s = r.t_submit;
    info->start_s = r.t_start;
    info->done_s = r.t_done;
    info->cell_updates = r.cells;
}

}  // namespace

extern "C" int sssi_plan_create(const sssi_plan_config* config, sssi_plan** plan) {
    return guarded([&] {
        SSSI_REQUIRE(config && plan, SSSI_ERR_ARG, "config and plan must not be NULL");
        const sssi_plan_config& c = *config;
        SSSI_REQUIRE(c.mode == SSSI_MODE_FP32 || c.mode == SSSI_MODE_FP64 || c.mode == SSSI_MODE_FP64_STRICT,
                     SSSI_ERR_ARG, "unknown mode %d", c.mode);
        SSSI_REQUIRE(c.nDiffOrder >= 1 && c.nDiffOrder <= kMaxOrder, SSSI_ERR_ARG, "nDiffOrder must be in 1..%d",
                     kMaxOrder);
        SSSI_REQUIRE(c.dz > 0 && c.dx > 0 && c.dy >= 0, SSSI_ERR_ARG, "dz and dx must be positive, dy >= 0");
        ensure_device();
        auto p = std::make_unique<sssi_plan>();
        p->cfg = c;
        if (p->cfg.mode == SSSI_MODE_FP64_STRICT) p->cfg.mode = SSSI_MODE_FP64;
        if (p->cfg.dy <= 0) p->cfg.dy = p->cfg.dx;
        SSSI_CHECK_CUDA(cudaGetDevice(&p->device));
        size_t free_b = 0, total_b = 0;
        SSSI_CHECK_CUDA(cudaMemGetInfo(&free_b, &total_b));
        p->budget = c.device_bytes ? c.device_bytes : free_b / 4 * 3;
        SSSI_CHECK_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
        SSSI_CHECK_CUDA(cudaStreamCreateWithFlags(&p->dstream, cudaStreamNonBlocking));
        p->t0 = Clock::now();
        if (p->cfg.mode == SSSI_MODE_FP32)
            p->engine = std::make_unique<Engine<float>>(p->cfg, p->stream);
        else
            p->engine = std::make_unique<Engine<double>>(p->cfg, p->stream);
        sssi_plan* raw = p.release();
        raw->deliverer = std::thread([raw] { raw->deliver_loop(); });
        raw->worker = std::thread([raw] { raw->run(); });
        *plan = raw;
    });
}

extern "C" int sssi_plan_destroy(sssi_plan* plan) {
    return guarded([&] {
        if (!plan) return;
        {
            std::lock_guard<std::mutex> lk(plan->mu);
            plan->stop = true;
        }
        plan->cv_work.notify_all();
        if (plan->worker.joinable()) plan->worker.join();
        {
            std::lock_guard<std::mutex> lk(plan->mu);
            plan->deliver_stop = true;
        }
        plan->cv_deliver.notify_all();
        if (plan->deliverer.joinable()) plan->deliverer.join();
        cudaStreamDestroy(plan->stream);
        cudaStreamDestroy(plan->dstream);
        delete plan;
    });
}

extern "C" int sssi_shot_submit(sssi_plan* plan, const sssi_shot_desc* shot, int64_t* ticket) {
    return guarded([&] {
        SSSI_REQUIRE(plan && shot && ticket, SSSI_ERR_ARG, "plan, shot and ticket must not be NULL");
        const sssi_shot_desc& d = *shot;
        SSSI_REQUIRE(d.kind == SSSI_SHOT_FWD2D || d.kind == SSSI_SHOT_RTM2D || d.kind == SSSI_SHOT_FWD3D,
                     SSSI_ERR_ARG, "unknown shot kind %d", d.kind);
        const bool is3 = d.kind == SSSI_SHOT_FWD3D;
        SSSI_REQUIRE(d.v && d.nz > 0 && d.nx > 0 && d.nt >= 0 && (!is3 || d.ny > 0), SSSI_ERR_ARG,
                     "bad shot sizes nz=%lld nx=%lld ny=%lld nt=%lld", (long long)d.nz, (long long)d.nx,
                     (long long)d.ny, (long long)d.nt);
        SSSI_REQUIRE(d.nBoundary >= 0 && d.nBoundary <= d.nz && 2 * (int64_t)d.nBoundary <= d.nx &&
                         (!is3 || 2 * (int64_t)d.nBoundary <= d.ny),
                     SSSI_ERR_ARG, "nBoundary %d does not fit the grid", d.nBoundary);
        SSSI_REQUIRE(d.dt > 0, SSSI_ERR_ARG, "dt must be positive");
        SSSI_REQUIRE(d.nt < (1LL << 30), SSSI_ERR_ARG, "nt too large");
        SSSI_REQUIRE(d.nsrc >= 0 && d.nsrc <= kMaxPointSources, SSSI_ERR_ARG, "nsrc must be in 0..%d", kMaxPointSources);
        SSSI_REQUIRE(d.nsrc == 0 || (d.src_iz && d.src_ix && d.wavelets && (!is3 || d.src_iy)), SSSI_ERR_ARG,
                     "point-source arrays are NULL");
        for (int s = 0; s < d.nsrc; ++s)
            SSSI_REQUIRE(d.src_iz[s] >= 0 && d.src_iz[s] < d.nz && d.src_ix[s] >= 0 && d.src_ix[s] < d.nx &&
                             (!is3 || (d.src_iy[s] >= 0 && d.src_iy[s] < d.ny)),
                         SSSI_ERR_ARG, "point source %d outside the grid", s);
        if (d.kind == SSSI_SHOT_RTM2D) {
            SSSI_REQUIRE(d.vs && (d.image || d.stack), SSSI_ERR_ARG, "RTM needs vs, and an image or a stack");
            SSSI_REQUIRE(d.nsrc == 1, SSSI_ERR_ARG, "RTM takes exactly one point source");
            SSSI_REQUIRE(d.snap_stride >= 0, SSSI_ERR_ARG, "snap_stride must be >= 0");
        }
        auto r = std::make_shared<PlanRequest>();
        r->d = d;
        const size_t n = (size_t)(d.nz * d.nx * (is3 ? d.ny : 1));
        r->v = api::host_copy(d.v, n, cudaStreamLegacy);
        if (d.kind == SSSI_SHOT_RTM2D) r->vs = api::host_copy(d.vs, n, cudaStreamLegacy);
        if (d.nsrc) r->wav = api::host_copy(d.wavelets, (size_t)(d.nsrc * d.nt), cudaStreamLegacy);
        r->iz.assign(d.src_iz, d.src_iz + d.nsrc);
        r->ix.assign(d.src_ix, d.src_ix + d.nsrc);
        if (is3) r->iy.assign(d.src_iy, d.src_iy + d.nsrc);
        r->d.v = r->d.vs = r->d.wavelets = nullptr;  // the copies are used from here on
        r->d.src_iz = r->d.src_ix = r->d.src_iy = nullptr;
        r->bytes = plan->engine->footprint(*r);
        {
            std::lock_guard<std::mutex> lk(plan->mu);
            SSSI_REQUIRE(!plan->stop, SSSI_ERR_ARG, "plan is being destroyed");
            if (d.stack) {
                SSSI_REQUIRE(d.kind == SSSI_SHOT_RTM2D, SSSI_ERR_ARG, "only RTM shots add to a stack");
                auto it = plan->stacks.find(d.stack);
                SSSI_REQUIRE(it != plan->stacks.end(), SSSI_ERR_ARG, "unknown stack %lld", (long long)d.stack);
                auto& st = *it->second;
                SSSI_REQUIRE(d.stack_z0 >= 0 && d.stack_x0 >= 0 && d.stack_z0 + d.nz <= st.nz &&
                                 d.stack_x0 + d.nx <= st.nx,
                             SSSI_ERR_ARG, "the shot's %lld x %lld grid at (%lld, %lld) leaves the %lld x %lld stack",
                             (long long)d.nz, (long long)d.nx, (long long)d.stack_z0, (long long)d.stack_x0,
                             (long long)st.nz, (long long)st.nx);
                r->stack_ptr = st.buf.as<double>() + d.stack_z0 + d.stack_x0 * st.nz;
                r->stack_ld = st.nz;
                ++st.pending;
            }
            r->ticket = plan->next_ticket++;
            r->t_submit = plan->now();
            plan->tickets[r->ticket] = r;
            plan->queue.push_back(r);
            *ticket = r->ticket;
        }
        plan->cv_work.notify_all();
    });
}

extern "C" int sssi_plan_stack_create(sssi_plan* plan, int64_t nz, int64_t nx, int64_t* stack) {
    return guarded([&] {
        SSSI_REQUIRE(plan && stack, SSSI_ERR_ARG, "plan and stack must not be NULL");
        SSSI_REQUIRE(nz > 0 && nx > 0 && nz < (int64_t(1) << 30) && nx < (int64_t(1) << 30), SSSI_ERR_ARG,
                     "bad stack size %lld x %lld", (long long)nz, (long long)nx);
        int dev = 0;
        SSSI_CHECK_CUDA(cudaGetDevice(&dev));
        SSSI_REQUIRE(dev == plan->device, SSSI_ERR_ARG, "the plan lives on device %d, the calling thread uses %d",
                     plan->device, dev);
        auto st = std::make_unique<sssi_plan::Stack>();
        st->nz = nz;
        st->nx = nx;
        st->buf.allocate(sizeof(double) * (size_t)(nz * nx));
        st->buf.zero(plan->stream);  // the worker's stream: ordered before any shot adds to it
        SSSI_CHECK_CUDA(cudaStreamSynchronize(plan->stream));
        std::lock_guard<std::mutex> lk(plan->mu);
        plan->in_use += st->buf.bytes();
        *stack = plan->next_stack++;
        plan->stacks[*stack] = std::move(st);
    });
}

extern "C" int sssi_plan_stack_get(sssi_plan* plan, int64_t stack, double* out) {
    return guarded([&] {
        SSSI_REQUIRE(plan && out, SSSI_ERR_ARG, "plan and out must not be NULL");
        std::unique_lock<std::mutex> lk(plan->mu);
        auto it = plan->stacks.find(stack);
        SSSI_REQUIRE(it != plan->stacks.end(), SSSI_ERR_ARG, "unknown stack %lld", (long long)stack);
        sssi_plan::Stack& st = *it->second;
        plan->cv_done.wait(lk, [&] { return st.pending == 0; });
        // every contribution's kernel ran before its shot was reported finished
        SSSI_CHECK_CUDA(cudaMemcpy(out, st.buf.get(), sizeof(double) * (size_t)(st.nz * st.nx), cudaMemcpyDefault));
    });
}

extern "C" int sssi_cancel(sssi_plan* plan, int64_t ticket) {
    return guarded([&] {
        SSSI_REQUIRE(plan, SSSI_ERR_ARG, "plan is NULL");
        std::lock_guard<std::mutex> lk(plan->mu);
        auto it = plan->tickets.find(ticket);
        SSSI_REQUIRE(it != plan->tickets.end(), SSSI_ERR_ARG, "unknown ticket %lld", (long long)ticket);
        ReqPtr r = it->second;
        if (r->state == SSSI_SHOT_QUEUED) {
            // not admitted yet: it leaves the queue now
            for (auto q = plan->queue.begin(); q != plan->queue.end(); ++q)
                if (q->get() == r.get()) {
                    plan->queue.erase(q);
                    break;
                }
            r->status = SSSI_ERR_CANCELLED;
            r->msg = "cancelled";
            r->state = SSSI_SHOT_FAILED;
            r->t_done = plan->now();
            ++plan->n_failed;
            if (r->d.stack) {
                auto st = plan->stacks.find(r->d.stack);
                if (st != plan->stacks.end()) --st->second->pending;
            }
            plan->cv_done.notify_all();
        } else if (r->state == SSSI_SHOT_RUNNING) {
            r->cancel.store(true);  // the worker drops it at its next round
            plan->cv_work.notify_all();
        }
    });
}

extern "C" int sssi_poll(sssi_plan* plan, int64_t ticket, sssi_shot_info* info) {
    return guarded([&] {
        SSSI_REQUIRE(plan, SSSI_ERR_ARG, "plan is NULL");
        std::lock_guard<std::mutex> lk(plan->mu);
        auto it = plan->tickets.find(ticket);
        SSSI_REQUIRE(it != plan->tickets.end(), SSSI_ERR_ARG, "unknown ticket %lld", (long long)ticket);
        fill_info(*it->second, info);
    });
}

extern "C" int sssi_wait(sssi_plan* plan, int64_t ticket, sssi_shot_info* info) {
    int status = SSSI_OK;
    std::string msg;
    const int rc = guarded([&] {
        SSSI_REQUIRE(plan, SSSI_ERR_ARG, "plan is NULL");
        std::unique_lock<std::mutex> lk(plan->mu);
        auto it = plan->tickets.find(ticket);
        SSSI_REQUIRE(it != plan->tickets.end(), SSSI_ERR_ARG, "unknown ticket %lld", (long long)ticket);
        ReqPtr r = it->second;
        plan->cv_done.wait(lk, [&] { return r->state == SSSI_SHOT_DONE || r->state == SSSI_SHOT_FAILED; });
        fill_info(*r, info);
        status = r->status;
        msg = r->msg;
    });
    if (rc != SSSI_OK) return rc;
    if (status != SSSI_OK) set_error("shot %lld failed: %s", (long long)ticket, msg.c_str());
    return status;
}

extern "C" int sssi_plan_stats_get(sssi_plan* plan, sssi_plan_stats* stats) {
    return guarded([&] {
        SSSI_REQUIRE(plan && stats, SSSI_ERR_ARG, "plan and stats must not be NULL");
        std::lock_guard<std::mutex> lk(plan->mu);
        stats->queued = (int64_t)plan->queue.size();
        stats->running = plan->n_running;
        stats->done = plan->n_done;
        stats->failed = plan->n_failed;
        stats->device_bytes_in_use = plan->in_use;
        stats->device_bytes_budget = plan->budget;
        stats->batch_steps = plan->batch_steps;
        stats->cell_updates = plan->cells;
        stats->admit_s = plan->admit_s;
        stats->round_s = plan->round_s;
        stats->gpu_wait_s = plan->gpu_wait_s;
        stats->batch2d_gpu_s = plan->batch2d_gpu_s;
        stats->batch2d_cell_updates = plan->batch2d_cells;
        stats->batch2d_tile_shape = plan->tile_shape;
        for (int v = 0; v < 3; ++v) stats->batch2d_tune_ms[v] = plan->tune_ms[v];
        stats->deliver_s = plan->deliver_s;
    });
}
