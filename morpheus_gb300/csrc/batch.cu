// Batched and served proving of many independent instances.
//
// An instance is d multilinear polynomials p_0..p_{d-1} over n variables, proven as
//   1. Basefold commit of every p_j (roots),
//   2. the product sumcheck of prod_j p_j over {0,1}^n with Ext2 challenges
//      (GpuLinearSumcheckProver, zk-torch-3/src/sumcheck/gpu_prover.rs:21-89), on the transcript
//      Transcript::new("sumcheck") . append_ext2("", master_seed) . append_u64("", index)
//      . append_u64("", root words of p_0..p_{d-1}),
//   3. Basefold open_ext2 of every p_j at the sumcheck point, each on its own transcript
//      Transcript::new("bf-open") . append_ext2("", master_seed) . append_u64("", 8 index + j),
//      the per-opening transcript of the reference's DAG prover (zk-torch-3/src/dag/mod.rs:1128-1133).
// Every transcript belongs to one instance, so an instance's proof does not depend on which
// other instances run beside it.
//
// The prover service runs instances on a pool of host worker threads, each launching on a
// stream of its own, so that the kernels of concurrent instances overlap on the device and
// one instance's host round trips (transcript challenges between rounds) hide behind the
// others' kernels.  The reference's DAG prover uses the same shape for its GPU openings
// (a rayon pool of GPU_OPEN_THREADS_PER_DEVICE = 12 threads per device, largest task first,
// zk-torch-3/src/dag/mod.rs:1102-1117).  Jobs are admitted against an HBM budget: a job
// starts when its estimated device footprint fits beside the running ones (the first queued
// job that fits, in arrival order; a job larger than the whole budget runs alone).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"
#include "common.cuh"
#include "host_field.hpp"
#include "open_engine.cuh"

namespace gb {

int matmul_prologue(void* table, void* ajtai_key, const u64 seed[2], int q, const gb_matmul_job* job,
                    std::vector<OpenTask>* tasks, std::vector<void*>* coms);

constexpr int INST_MAX_D = 8;
constexpr int INST_LOG_RATE = 1;

static size_t inst_proof_len(int n, int d, int q) {
    size_t sc = (size_t)n * (d + 1) * 2 + (size_t)n * 2 + (size_t)d * 2 + 2;
    return (size_t)d * 4 + sc + (size_t)d * gb_basefold_proof_len(n, INST_LOG_RATE, q);
}

// Device bytes one instance holds at its peak: inputs and d commitments (evaluation copy,
// codeword, tree), the sumcheck's two Ext2 levels, and one opening's workspace.
static size_t inst_hbm_bytes(int n, int d) {
    size_t N = (size_t)1 << n;
    return N * ((size_t)d * (8 + 8 + 16 + 64 + 16) + 144) + ((size_t)1 << 20);
}

using Clock = std::chrono::steady_clock;
static double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Everything of one instance before its openings, on the calling thread's stream: the commits
// and the product sumcheck.  On success the commitments (handles in *coms) and one OpenTask per
// polynomial (its point, its "bf-open" transcript preamble, its place in the proof) are returned
// and the stream is idle; the caller opens and then destroys the commitments.
static int instance_prologue(void* table, const u64 seed[2], int q, const gb_instance* in,
                             std::vector<OpenTask>* tasks, std::vector<void*>* coms) {
    using namespace host;
    if (!table || !in || in->num_vars < 2 || in->num_vars > 30 || in->degree < 1 || in->degree > INST_MAX_D ||
        (!in->h_polys == !in->d_polys) || !in->h_proof || q < 0) {
        set_error_msg("gb_prove_instance: invalid argument");
        return GB_EINVAL;
    }
    const int n = in->num_vars, d = in->degree;
    cudaStream_t s = stream();
    const size_t N = (size_t)1 << n;
    const u64* polys = in->d_polys;
    u64* owned = nullptr;
    if (in->h_polys) {
        GB_CUDA_TRY(cudaMallocAsync(&owned, N * d * 8, s));
        cudaError_t e = cudaMemcpyAsync(owned, in->h_polys, N * d * 8, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(owned, s);
            set_error("cudaMemcpyAsync", e);
            return GB_ECUDA;
        }
        polys = owned;
    }
    u64* out = in->h_proof;
    u64* roots = out;
    u64* msgs = roots + (size_t)d * 4;
    u64* chal = msgs + (size_t)n * (d + 1) * 2;
    u64* finals = chal + (size_t)n * 2;
    u64* final_eval = finals + (size_t)d * 2;
    u64* opens = final_eval + 2;
    const size_t plen = gb_basefold_proof_len(n, INST_LOG_RATE, q);

    std::vector<void*> com(d, nullptr);
    int rc = GB_OK;
    for (int j = 0; j < d && !rc; j++)
        rc = gb_basefold_commit(polys + (size_t)j * N, nullptr, n, INST_LOG_RATE, &com[j], roots + 4 * j);
    if (!rc) {
        gb_transcript t;
        gb_transcript_new(&t, "sumcheck");
        tr_append_ext2(&t, "", E2{canon(seed[0]), canon(seed[1])});
        tr_append_u64(&t, "", in->index);
        for (int k = 0; k < 4 * d; k++) tr_append_u64(&t, "", roots[k]);
        rc = gb_sumcheck_prove_ext2(&t, n, d, polys, nullptr, msgs, chal, finals, final_eval);
    }
    if (owned) cudaFreeAsync(owned, s);  // the commitments hold their own copies
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("cudaStreamSynchronize", e);
            rc = GB_ECUDA;
        }
    }
    if (rc) {
        for (int j = 0; j < d; j++)
            if (com[j]) gb_basefold_commitment_destroy(com[j]);
        return rc;
    }
    for (int j = 0; j < d; j++) {
        OpenTask t;
        t.com = (BfCommitment*)com[j];
        t.point.assign(chal, chal + 2 * (size_t)n);
        gb_transcript_new(&t.t, "bf-open");
        tr_append_ext2(&t.t, "", E2{canon(seed[0]), canon(seed[1])});
        tr_append_u64(&t.t, "", 8 * in->index + (u64)j);
        t.proof = opens + (size_t)j * plen;
        tasks->push_back(std::move(t));
        coms->push_back(com[j]);
    }
    return GB_OK;
}

int open_tasks_inline(void* table, int q, std::vector<OpenTask>& tasks, std::vector<void*>& coms) {
    int rc = GB_OK;
    for (size_t k = 0; k < tasks.size() && !rc; k++)
        rc = gb_basefold_open_ext2(coms[k], table, tasks[k].point.data(), &tasks[k].t, q, tasks[k].proof);
    for (void* c : coms) gb_basefold_commitment_destroy(c);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(stream());
        if (e != cudaSuccess) {
            set_error("cudaStreamSynchronize", e);
            rc = GB_ECUDA;
        }
    }
    return rc;
}

// Prove one instance on the calling thread's stream.
static int prove_instance(void* table, const u64 seed[2], int q, const gb_instance* in) {
    std::vector<OpenTask> tasks;
    std::vector<void*> coms;
    int rc = instance_prologue(table, seed, q, in, &tasks, &coms);
    if (rc) return rc;
    return open_tasks_inline(table, q, tasks, coms);
}

// ---------------------------------------------------------------------------
// prover service
// ---------------------------------------------------------------------------
struct Job {
    int kind = 0;  // 0: instance, 1: matmul layer
    gb_instance inst;
    gb_matmul_job mm;
    uint64_t ticket = 0;
    size_t bytes = 0;
    int rc = 0;
    bool done = false;
    Clock::time_point submitted, started, finished;
    std::string err;
};

// Two modes.  Whole-job: a worker runs a job from start to end on its stream.  Continuous: a
// worker runs a job's prologue (inputs, commits, sumcheck, partial evaluations, Ajtai) on its
// stream and hands the job's openings to the service's open engines, which batch them with the
// openings of every other job in flight round by round (open_engine.cuh); the worker then takes
// the next admitted job, and the job completes, and frees its share of the budget, when its
// last opening leaves its engine.  There is one engine (thread and stream) per size class of
// openings, so that a step of small openings does not wait for a large opening's round (a
// 2^24-evaluation opening's first tree takes ~9 ms of permutations; a 2^16 one's whole opening
// ~0.1 ms), and the classes' steps overlap on the device.
constexpr int OPEN_CLASS_CUTS[] = {19, 22};  // classes n < 19, 19 <= n < 22, n >= 22
constexpr int OPEN_CLASSES = 3;
static int open_class(int n) {
    int c = 0;
    while (c < OPEN_CLASSES - 1 && n >= OPEN_CLASS_CUTS[c]) c++;
    return c;
}

class Prover {
  public:
    Prover(void* table, const u64 seed[2], int q, int workers, size_t budget, int device, bool continuous)
        : table_(table), q_(q), budget_(budget), device_(device) {
        seed_[0] = seed[0];
        seed_[1] = seed[1];
        if (continuous)
            for (int c = 0; c < OPEN_CLASSES && !start_rc_; c++) {
                int rc = GB_OK;
                OpenEngine* e = open_engine_create((const BfTable*)table, q, device, &rc);
                if (!e) start_rc_ = rc ? rc : GB_EINVAL;
                else engines_.push_back(e);
            }
        for (int w = 0; w < workers; w++) threads_.emplace_back([this] { run(); });
    }
    ~Prover() {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        for (auto& t : threads_) t.join();
        for (OpenEngine* e : engines_) open_engine_destroy(e);  // finishes the openings in flight
    }
    int start_error() {
        std::unique_lock<std::mutex> l(mu_);
        cv_done_.wait(l, [this] { return ready_ == (int)threads_.size(); });
        return start_rc_;
    }
    void set_coop(size_t v) { coop_.store(v); }
    void set_top(size_t v) { top_.store(v); }
    void set_slots(int k) {
        {
            std::lock_guard<std::mutex> l(mu_);
            slots_ = k;
        }
        cv_work_.notify_all();
    }
    void set_ajtai_key(void* key) {
        std::lock_guard<std::mutex> l(mu_);
        ajtai_key_ = key;
    }
    uint64_t submit(const gb_instance& in) {
        auto j = std::make_unique<Job>();
        j->inst = in;
        j->bytes = inst_hbm_bytes(in.num_vars, in.degree);
        return enqueue(std::move(j));
    }
    uint64_t submit(const gb_matmul_job& mm) {
        auto j = std::make_unique<Job>();
        j->kind = 1;
        j->mm = mm;
        j->bytes = gb_matmul_hbm_bytes(mm.m, mm.n, mm.k);
        return enqueue(std::move(j));
    }
    uint64_t enqueue(std::unique_ptr<Job> j) {
        j->submitted = Clock::now();
        std::lock_guard<std::mutex> l(mu_);
        j->ticket = ++next_ticket_;
        uint64_t t = j->ticket;
        queue_.push_back(j.get());
        jobs_.emplace(t, std::move(j));
        cv_work_.notify_one();
        return t;
    }
    int wait(uint64_t ticket, gb_job_stats* st) {
        std::unique_lock<std::mutex> l(mu_);
        auto it = jobs_.find(ticket);
        if (it == jobs_.end()) {
            set_error_msg("gb_prover_wait: unknown ticket");
            return GB_EINVAL;
        }
        Job* j = it->second.get();
        cv_done_.wait(l, [j] { return j->done; });
        if (st) {
            st->queued_ms = ms_between(j->submitted, j->started);
            st->run_ms = ms_between(j->started, j->finished);
            st->latency_ms = ms_between(j->submitted, j->finished);
        }
        int rc = j->rc;
        if (rc) set_error_msg(j->err);
        jobs_.erase(it);
        return rc;
    }
    int drain() {
        std::unique_lock<std::mutex> l(mu_);
        cv_done_.wait(l, [this] { return queue_.empty() && running_ == 0; });
        return GB_OK;
    }
    size_t engine_in_flight() {
        size_t k = 0;
        for (OpenEngine* e : engines_) k += open_engine_in_flight(e);
        return k;
    }
    // jobs admitted and not yet complete (in a prologue or with openings in an engine)
    int running() {
        std::lock_guard<std::mutex> l(mu_);
        return running_;
    }

  private:
    // the first queued job that fits the budget beside the running ones; a job larger than
    // the whole budget is taken only when nothing runs
    Job* take_locked() {
        if (slots_ > 0 && running_ >= slots_) return nullptr;  // every slot holds a job in flight
        for (auto it = queue_.begin(); it != queue_.end(); ++it) {
            Job* j = *it;
            if (in_use_ + j->bytes <= budget_ || running_ == 0) {
                queue_.erase(it);
                return j;
            }
        }
        return nullptr;
    }
    void run() {
        cudaStream_t st = nullptr;
        int rc = cudaSetDevice(device_) == cudaSuccess &&
                         cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess
                     ? GB_OK
                     : GB_ECUDA;
        if (!rc) gb_set_stream(st);
        {
            std::lock_guard<std::mutex> l(mu_);
            if (rc) start_rc_ = rc;
            ready_++;
        }
        cv_done_.notify_all();
        for (;;) {
            Job* j = nullptr;
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_work_.wait(l, [&] { return stop_ || (j = take_locked()) != nullptr; });
                if (!j) break;
                in_use_ += j->bytes;
                running_++;
                j->started = Clock::now();
            }
            gb_set_coop_threshold(coop_.load());
            gb_set_merkle_top_nodes(top_.load());
            if (!engines_.empty() && !rc) {
                std::vector<OpenTask> tasks;
                std::vector<void*> coms;
                int prc = j->kind == 0 ? instance_prologue(table_, seed_, q_, &j->inst, &tasks, &coms)
                                       : matmul_prologue(table_, ajtai_key_, seed_, q_, &j->mm, &tasks, &coms);
                if (!prc) hand_to_engines(j, tasks, coms);
                else complete(j, prc, gb_last_error());
                continue;
            }
            int jrc = rc ? rc
                      : j->kind == 0 ? prove_instance(table_, seed_, q_, &j->inst)
                                     : gb_prove_matmul(table_, ajtai_key_, seed_, q_, &j->mm);
            complete(j, jrc, jrc ? std::string(gb_last_error()) : std::string());
        }
        if (st) {
            cudaStreamSynchronize(st);
            gb_set_stream(nullptr);
            cudaStreamDestroy(st);
        }
    }

    void complete(Job* j, int rc, const std::string& err) {
        {
            std::lock_guard<std::mutex> l(mu_);
            j->finished = Clock::now();
            j->rc = rc;
            j->err = err;
            j->done = true;
            in_use_ -= j->bytes;
            running_--;
        }
        cv_done_.notify_all();
        cv_work_.notify_all();  // freed budget may admit a waiting job
    }
    // the job's openings into the engines of their size classes; the last one to finish
    // completes the job (on an engine thread)
    void hand_to_engines(Job* j, std::vector<OpenTask>& tasks, std::vector<void*>& coms) {
        struct Pending {
            std::mutex mu;
            int left = 0, rc = GB_OK;
            std::string err;
        };
        auto pend = std::make_shared<Pending>();
        pend->left = (int)tasks.size();
        for (size_t k = 0; k < tasks.size(); k++) {
            void* com = coms[k];
            OpenEngine* e = engines_[open_class(tasks[k].com->num_vars)];
            tasks[k].done = [this, j, pend, com](int rc, const std::string& err) {
                gb_basefold_commitment_destroy(com);
                bool last;
                {
                    std::lock_guard<std::mutex> l(pend->mu);  // the engines are separate threads
                    if (rc && !pend->rc) {
                        pend->rc = rc;
                        pend->err = err;
                    }
                    last = --pend->left == 0;
                }
                if (last) complete(j, pend->rc, pend->err);
            };
            open_engine_submit(e, std::move(tasks[k]));
        }
    }

    void* table_;
    void* ajtai_key_ = nullptr;
    std::vector<OpenEngine*> engines_;  // continuous mode: one per size class
    std::atomic<size_t> coop_{gb_get_coop_threshold()};
    std::atomic<size_t> top_{gb_get_merkle_top_nodes()};
    u64 seed_[2];
    int q_;
    size_t budget_;
    int device_;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<Job*> queue_;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs_;
    std::vector<std::thread> threads_;
    uint64_t next_ticket_ = 0;
    size_t in_use_ = 0;
    int slots_ = 0;  // jobs in flight at most (0: the budget alone limits them)
    int running_ = 0, ready_ = 0, start_rc_ = 0;
    bool stop_ = false;
};

}  // namespace gb

using namespace gb;

extern "C" {

size_t gb_instance_proof_len(int num_vars, int degree, int num_queries) {
    return inst_proof_len(num_vars, degree, num_queries);
}

size_t gb_instance_hbm_bytes(int num_vars, int degree) { return inst_hbm_bytes(num_vars, degree); }

int gb_prove_instance(void* table, const uint64_t master_seed[2], int num_queries, const gb_instance* inst) {
    if (!master_seed) return GB_EINVAL;
    return prove_instance(table, master_seed, num_queries, inst);
}

static int prover_create(void* table, const uint64_t master_seed[2], int num_queries, int workers, size_t hbm_budget,
                         bool continuous, void** handle) {
    if (!table || !master_seed || !handle || workers < 1 || workers > 256 || num_queries < 0 ||
        (continuous && ((const BfTable*)table)->log_rate != 1)) {
        set_error_msg("gb_prover_create: invalid argument (the continuous service needs a log_rate 1 table)");
        return GB_EINVAL;
    }
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    Prover* p = new Prover(table, master_seed, num_queries, workers, hbm_budget, dev, continuous);
    int rc = p->start_error();
    if (rc) {
        delete p;
        set_error_msg("gb_prover_create: a worker or an open engine could not start");
        return rc;
    }
    *handle = p;
    return GB_OK;
}

int gb_prover_create(void* table, const uint64_t master_seed[2], int num_queries, int workers, size_t hbm_budget,
                     void** handle) {
    return prover_create(table, master_seed, num_queries, workers, hbm_budget, false, handle);
}

int gb_prover_create_continuous(void* table, const uint64_t master_seed[2], int num_queries, int workers,
                                size_t hbm_budget, void** handle) {
    return prover_create(table, master_seed, num_queries, workers, hbm_budget, true, handle);
}

int gb_prover_running(void* prover) { return prover ? static_cast<Prover*>(prover)->running() : -1; }

size_t gb_prover_openings_in_flight(void* prover) {
    return prover ? static_cast<Prover*>(prover)->engine_in_flight() : 0;
}

int gb_prover_submit(void* prover, const gb_instance* inst, uint64_t* ticket) {
    if (!prover || !inst || !ticket) return GB_EINVAL;
    const int n = inst->num_vars, d = inst->degree;
    if (n < 2 || n > 30 || d < 1 || d > INST_MAX_D || (!inst->h_polys == !inst->d_polys) || !inst->h_proof) {
        set_error_msg("gb_prover_submit: invalid instance");
        return GB_EINVAL;
    }
    *ticket = static_cast<Prover*>(prover)->submit(*inst);
    return GB_OK;
}

int gb_prover_set_coop_threshold(void* prover, size_t parents) {
    if (!prover) return GB_EINVAL;
    static_cast<Prover*>(prover)->set_coop(parents);
    return GB_OK;
}

int gb_prover_set_merkle_top_nodes(void* prover, size_t nodes) {
    if (!prover) return GB_EINVAL;
    static_cast<Prover*>(prover)->set_top(nodes);
    return GB_OK;
}

int gb_prover_set_slots(void* prover, int slots) {
    if (!prover || slots < 0) return GB_EINVAL;
    static_cast<Prover*>(prover)->set_slots(slots);
    return GB_OK;
}

int gb_prover_set_ajtai_key(void* prover, void* ajtai_key) {
    if (!prover || !ajtai_key) return GB_EINVAL;
    static_cast<Prover*>(prover)->set_ajtai_key(ajtai_key);
    return GB_OK;
}

int gb_prover_submit_matmul(void* prover, const gb_matmul_job* job, uint64_t* ticket) {
    if (!prover || !job || !ticket) return GB_EINVAL;
    if (gb_matmul_proof_len(job->m, job->n, job->k, 0) == 0 || !job->h_a || !job->h_b || !job->h_proof) {
        set_error_msg("gb_prover_submit_matmul: invalid job");
        return GB_EINVAL;
    }
    *ticket = static_cast<Prover*>(prover)->submit(*job);
    return GB_OK;
}

int gb_prover_wait(void* prover, uint64_t ticket, gb_job_stats* stats) {
    if (!prover) return GB_EINVAL;
    return static_cast<Prover*>(prover)->wait(ticket, stats);
}

int gb_prover_drain(void* prover) {
    if (!prover) return GB_EINVAL;
    return static_cast<Prover*>(prover)->drain();
}

int gb_prover_destroy(void* prover) {
    if (!prover) return GB_EINVAL;
    delete static_cast<Prover*>(prover);
    return GB_OK;
}

int gb_batch_prove(void* table, const uint64_t master_seed[2], int num_queries, const gb_instance* insts, int count,
                   int workers, size_t hbm_budget) {
    if (count < 0 || (count > 0 && !insts)) return GB_EINVAL;
    if (count == 0) return GB_OK;
    void* h = nullptr;
    int rc = gb_prover_create(table, master_seed, num_queries, workers, hbm_budget, &h);
    if (rc) return rc;
    // largest instance first: the long ones start early and the small ones fill in behind
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return inst_hbm_bytes(insts[a].num_vars, insts[a].degree) > inst_hbm_bytes(insts[b].num_vars, insts[b].degree);
    });
    std::vector<uint64_t> tickets(count, 0);
    for (int k = 0; k < count && !rc; k++) rc = gb_prover_submit(h, &insts[order[k]], &tickets[k]);
    int first = rc;
    std::string msg = rc ? std::string(gb_last_error()) : std::string();
    for (int k = 0; k < count; k++) {
        if (!tickets[k]) continue;
        int r = gb_prover_wait(h, tickets[k], nullptr);
        if (r && !first) {
            first = r;
            msg = gb_last_error();
        }
    }
    gb_prover_destroy(h);
    if (first) set_error_msg(msg);
    return first;
}

}  // extern "C"
