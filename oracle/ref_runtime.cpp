// ref_runtime.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's compute shaders (compiled as C++ by ref_build.py) the
// way a GPU runs a dispatch: workgroup by workgroup, each invocation of a
// workgroup a fiber (ucontext) with its own stack.  barrier() suspends the
// invocation; once every live invocation of the workgroup is suspended at the
// barrier (or finished) they all resume.  Invocations run in id order between
// barriers, so results are deterministic.
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ref_shim.h"

uvec3 gl_GlobalInvocationID;
uvec3 gl_LocalInvocationID;
uvec3 gl_WorkGroupID;
vec4 gl_Position;
vec3 ref_dfdx;
vec3 ref_dfdy;

namespace {

constexpr size_t kStack = 256 * 1024;

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    bool done = false;
};

ucontext_t g_sched;
Fiber* g_cur = nullptr;
void (*g_main)() = nullptr;
bool g_flat = false;

void fiber_entry()
{
    g_main();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

}  // namespace

void ref_barrier()
{
    if (g_flat) {
        std::fprintf(stderr, "ref_runtime: barrier() in a program dispatched without fibers\n");
        std::abort();
    }
    if (!g_cur) return;  // workgroup of one invocation
    swapcontext(&g_cur->ctx, &g_sched);
}

void ref_dispatch(void (*main_fn)(), uvec3 groups, uint invocations)
{
    g_main = main_fn;
    if (invocations == 1) {  // no barrier can matter: plain calls
        g_cur = nullptr;
        for (uint z = 0; z < groups.z; ++z)
            for (uint y = 0; y < groups.y; ++y)
                for (uint x = 0; x < groups.x; ++x) {
                    gl_WorkGroupID = uvec3(x, y, z);
                    gl_LocalInvocationID = uvec3(0u);
                    gl_GlobalInvocationID = gl_WorkGroupID;
                    main_fn();
                }
        return;
    }
    std::vector<Fiber> fibers(invocations);
    for (auto& f : fibers) f.stack.resize(kStack);
    for (uint z = 0; z < groups.z; ++z)
        for (uint y = 0; y < groups.y; ++y)
            for (uint x = 0; x < groups.x; ++x) {
                for (uint i = 0; i < invocations; ++i) {
                    Fiber& f = fibers[i];
                    f.done = false;
                    getcontext(&f.ctx);
                    f.ctx.uc_stack.ss_sp = f.stack.data();
                    f.ctx.uc_stack.ss_size = f.stack.size();
                    f.ctx.uc_link = nullptr;
                    makecontext(&f.ctx, fiber_entry, 0);
                }
                const uvec3 wg(x, y, z);
                for (;;) {
                    uint live = 0;
                    for (uint i = 0; i < invocations; ++i) {
                        Fiber& f = fibers[i];
                        if (f.done) continue;
                        gl_WorkGroupID = wg;
                        gl_LocalInvocationID = uvec3(i, 0u, 0u);
                        gl_GlobalInvocationID = uvec3(x * invocations + i, y, z);
                        g_cur = &f;
                        swapcontext(&g_sched, &f.ctx);
                        if (!f.done) ++live;
                    }
                    if (live == 0) break;
                }
                g_cur = nullptr;
            }
}

void ref_dispatch_flat(void (*main_fn)(), uvec3 groups, uint invocations)
{
    g_cur = nullptr;
    g_flat = true;
    for (uint z = 0; z < groups.z; ++z)
        for (uint y = 0; y < groups.y; ++y)
            for (uint x = 0; x < groups.x; ++x)
                for (uint i = 0; i < invocations; ++i) {
                    gl_WorkGroupID = uvec3(x, y, z);
                    gl_LocalInvocationID = uvec3(i, 0u, 0u);
                    gl_GlobalInvocationID = uvec3(x * invocations + i, y, z);
                    main_fn();
                }
    g_flat = false;
}
