// ref_runtime.cpp — TEST INFRASTRUCTURE.  Work-group emulator for running the
// reference's OpenCL kernels on the host: every work-item of a group is a
// ucontext fiber; barrier() switches back to the group scheduler, which
// resumes the items round-robin until all of them have returned.
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "clshim.hpp"

namespace clshim {

thread_local WorkItem g_item;

namespace {
struct Fiber {
    ucontext_t ctx;
    WorkItem item;
    bool done = false;
};
thread_local ucontext_t t_sched;
thread_local Fiber* t_current = nullptr;
thread_local const std::function<void()>* t_body = nullptr;

void fiber_entry() {
    (*t_body)();
    t_current->done = true;
    // returning resumes uc_link (the scheduler)
}
}  // namespace

void barrier_impl() {
    if (!t_current) return;  // flat launch: barriers are no-ops
    Fiber* me = t_current;
    swapcontext(&me->ctx, &t_sched);
    g_item = me->item;
}

void launch_groups(size_t global, size_t local, const std::function<void()>& f) {
    const size_t stack_bytes = 64 * 1024;
    std::vector<Fiber> fibers(local);
    std::vector<char> stacks(stack_bytes * local);
    t_body = &f;
    for (size_t g0 = 0; g0 < global; g0 += local) {
        for (size_t l = 0; l < local; ++l) {
            Fiber& fb = fibers[l];
            fb.done = false;
            fb.item = WorkItem{g0 + l, l, g0 / local, local, global};
            getcontext(&fb.ctx);
            fb.ctx.uc_stack.ss_sp = &stacks[l * stack_bytes];
            fb.ctx.uc_stack.ss_size = stack_bytes;
            fb.ctx.uc_link = &t_sched;
            makecontext(&fb.ctx, fiber_entry, 0);
        }
        bool live = true;
        while (live) {
            live = false;
            for (size_t l = 0; l < local; ++l) {
                Fiber& fb = fibers[l];
                if (fb.done) continue;
                t_current = &fb;
                g_item = fb.item;
                swapcontext(&t_sched, &fb.ctx);
                if (!fb.done) live = true;
            }
        }
        t_current = nullptr;
    }
    t_body = nullptr;
}

}  // namespace clshim
