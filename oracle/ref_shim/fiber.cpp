/*
 * fiber.cpp -- cooperative CUDA-block emulation for the reference kernels.
 *
 * TEST INFRASTRUCTURE ONLY (oracle recipe).  A launch runs its blocks one
 * after another; the threads of a block are ucontext fibers.  A fiber runs
 * until it reaches a barrier (__syncthreads / __all_sync) or returns.  When
 * every live fiber of the block waits at a barrier, the scheduler resolves it
 * (for __all_sync: the AND of the predicates of the live fibers, which are the
 * active lanes) and resumes the fibers in thread order.  Resuming in thread
 * order is what makes the reference's warp-shared traversal stack correct
 * here: in Kernels.cu:522-566 every push by lane 0 happens right after a vote,
 * before any lane pops again.
 */
#include "cuda.h"

#include <functional>
#include <stdexcept>
#include <stdlib.h>
#include <ucontext.h>
#include <vector>

struct nbx_fiber {
    nbx_dim3 tid;
    ucontext_t ctx;
    int state; /* 0 runnable, 1 waiting at barrier, 2 finished */
    int kind;  /* 1 syncthreads, 2 all_sync */
    int pred, result;
    std::vector<char> stack;
};

nbx_fiber *nbx_cur_fiber = nullptr;
nbx_dim3 nbx_block_idx, nbx_block_dim, nbx_grid_dim;
static ucontext_t g_sched;
static std::function<void()> *g_body = nullptr;

nbx_dim3 &nbx_thread_idx() { return nbx_cur_fiber->tid; }

static void fiber_entry()
{
    (*g_body)();
    nbx_cur_fiber->state = 2;
    swapcontext(&nbx_cur_fiber->ctx, &g_sched);
}

static void wait_barrier(int kind, int pred)
{
    nbx_fiber *f = nbx_cur_fiber;
    f->state = 1;
    f->kind = kind;
    f->pred = pred;
    swapcontext(&f->ctx, &g_sched);
}

void nbx_syncthreads() { wait_barrier(1, 0); }

int nbx_all_sync(int pred)
{
    wait_barrier(2, pred);
    return nbx_cur_fiber->result;
}

/* Runs body() as <<<grid, block>>>; returns 0, or -1 on a barrier mismatch. */
int nbx_launch(int grid, int block, std::function<void()> body)
{
    g_body = &body;
    nbx_grid_dim = {(unsigned)grid, 1, 1};
    nbx_block_dim = {(unsigned)block, 1, 1};
    std::vector<nbx_fiber> fib(block);
    for (int b = 0; b < grid; b++) {
        nbx_block_idx = {(unsigned)b, 0, 0};
        for (int t = 0; t < block; t++) {
            nbx_fiber &f = fib[t];
            f.tid = {(unsigned)t, 0, 0};
            f.state = 0;
            f.stack.assign(256 * 1024, 0);
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = f.stack.data();
            f.ctx.uc_stack.ss_size = f.stack.size();
            f.ctx.uc_link = nullptr;
            makecontext(&f.ctx, fiber_entry, 0);
        }
        for (;;) {
            for (int t = 0; t < block; t++) {
                if (fib[t].state != 0) continue;
                nbx_cur_fiber = &fib[t];
                swapcontext(&g_sched, &fib[t].ctx);
            }
            int live = 0, kind = 0, all = 1;
            for (int t = 0; t < block; t++) {
                if (fib[t].state != 1) continue;
                if (live && fib[t].kind != kind) return -1;
                kind = fib[t].kind;
                all &= fib[t].pred;
                live++;
            }
            if (!live) break;
            for (int t = 0; t < block; t++) {
                if (fib[t].state != 1) continue;
                fib[t].result = all;
                fib[t].state = 0;
            }
        }
    }
    nbx_cur_fiber = nullptr;
    return 0;
}
