// Live continuous-batching MD serving: a library thread runs the serving loop of a
// session (Session::serve_loop, md_host.cu) while other threads submit requests and
// collect their results.  The session belongs to the server until stop().
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "session.h"

namespace cg {

// Status of poll() for a request that has not finished yet.
constexpr int CG_PENDING_STATUS = 5;

class MdServer : public ServeSource {
   public:
    // Starts the serving thread.  mass_type: one mass (amu) per atom type.
    MdServer(Session& s, const double* mass_type, const MdServeOptions& opt);
    ~MdServer() override;
    // Copies the request's inputs and queues it (arrival = now); returns its ticket.
    // Throws Error 1 / 2 for a request that can never run (bad input, more atoms than
    // the batch capacity, more device memory than the budget alone).
    int64_t submit(const MdRequest& q);
    // 0 and the result (and final positions, 3 per atom) once the request finished;
    // CG_PENDING_STATUS while it waits or runs (wait = false), or blocks until it
    // finishes (wait = true).  Throws the loop's error if the loop failed.
    int poll(int64_t ticket, bool wait, MdResult* r, double* xyz);
    // Stops taking requests, finishes every queued and running one, joins the thread;
    // returns the number of batched steps, or throws the loop's error.
    int64_t stop();

    // ServeSource (called by the serving thread)
    int next(double now) override;
    void admitted() override;
    const MdRequest& request(int id) override;
    bool wait(double now) override;
    void finished(int id, const MdResult& r) override;

   private:
    struct Ticket {
        MdRequest q;
        std::vector<int> types;
        std::vector<double> xyz, cell, v, out;
        MdResult res;
        bool done = false;
    };
    void run();
    Session& s_;
    std::vector<double> mass_;
    MdServeOptions opt_;
    std::mutex mu_;
    std::condition_variable cv_;   // new submissions, finished requests, the loop's end
    std::deque<Ticket> t_;
    size_t next_ = 0;              // first ticket not yet admitted
    bool stopping_ = false, ended_ = false;
    int err_code_ = 0;
    std::string err_msg_;
    int64_t steps_ = 0;
    std::thread th_;
};

}  // namespace cg
