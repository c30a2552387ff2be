// ngrav_gpu_accelfn.hpp -- the GB300 Barnes-Hut force evaluation as the
// reference's AccelFn<3> (include/ngrav/Integrator.hpp:13-14), for
// registration with System<3>::SetAuxSolver (include/ngrav/System.hpp:40).
//
// Header-only C++17 on top of the C-ABI (ngrav_gpu.h); it needs the
// reference's own headers (ngrav/Integrator.hpp and what it includes) on the
// include path and links -lngrav_gpu.  Each call copies the positions and
// masses in, evaluates on the GPU and writes out.ax/ay/az (G included), the
// contract of ComputeAccelBarnesHut(pts, sp, out)
// (include/ngrav/Solvers.hpp:56-57): `out` is resized, `in` may alias it.
// G, eps, the softening kind, theta and the MAC kind are taken from `sp` on
// every call.  A call whose particle count and masses equal the previous
// call's only moves the positions (ngrav_gpu_set_state), so the previous
// evaluation's |a| serves the relative opening test as its |a_old| -- the
// history System<3> keeps in m_aOldMag (CaptureAOld, System.hpp:302-310);
// any other call starts a new particle set without history, as
// System::SetParticles does.
//
// Copies share one GPU context (std::function copies its target, and
// System::SetAuxSolver stores a copy): a std::shared_ptr with
// ngrav_gpu_destroy as its deleter frees it when the last copy goes.
// Errors are thrown as std::runtime_error, the reference's error convention.
#pragma once

#include "ngrav/Integrator.hpp"
#include "ngrav_gpu.h"

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ngrav_gpu {

class GpuBarnesHut {
public:
    // leafCapacity: the reference's ncrit (AdaptiveTree's default 8);
    // device: the CUDA device of the context.
    explicit GpuBarnesHut(const ngrav::StepParams& sp, int leafCapacity = 8, int device = 0) {
        ngrav_gpu_opts o;
        ngrav_gpu_default_opts(&o);
        o.device = device;
        o.leaf_capacity = leafCapacity;
        Fill(o, sp);
        ngrav_gpu_ctx* raw = nullptr;
        const int rc = ngrav_gpu_create(&raw, &o);
        if (rc != NGRAV_OK) throw std::runtime_error("ngrav_gpu_create failed with status " + std::to_string(rc));
        m_ctx = std::shared_ptr<ngrav_gpu_ctx>(raw, ngrav_gpu_destroy);
        m_opts = o;
    }

    void operator()(const ngrav::SoA<3>& in, const ngrav::StepParams& sp, ngrav::SoA<3>& out) const {
        ngrav_gpu_ctx* ctx = m_ctx.get();
        ngrav_gpu_opts o = m_opts;
        Fill(o, sp);
        Check(ngrav_gpu_set_opts(ctx, &o));
        Check(ngrav_gpu_set_softening(ctx, sp.soft.kind == ngrav::SofteningKind::Spline ? NGRAV_SOFTENING_SPLINE
                                                                                         : NGRAV_SOFTENING_PLUMMER));
        if (sp.mac.kind == ngrav::MacKind::Relative) Check(ngrav_gpu_set_mac_alpha(ctx, sp.mac.alpha));
        const std::size_t n = in.Count();
        std::vector<double>& mass = *m_mass;
        if (n > 0 && n == mass.size() && std::equal(in.m.begin(), in.m.end(), mass.begin())) {
            Check(ngrav_gpu_set_state(ctx, in.x.data(), in.y.data(), in.z.data(), nullptr, nullptr, nullptr));
        } else {
            Check(ngrav_gpu_set_particles(ctx, (int64_t)n, in.x.data(), in.y.data(), in.z.data(), nullptr, nullptr,
                                          nullptr, in.m.data()));
            mass = in.m;
        }
        out.ResizeAccel(n);
        Check(ngrav_gpu_compute_accel(ctx, out.ax.data(), out.ay.data(), out.az.data()));
    }

    ngrav_gpu_ctx* Context() const { return m_ctx.get(); }

private:
    static void Fill(ngrav_gpu_opts& o, const ngrav::StepParams& sp) {
        o.G = sp.G;
        o.eps = sp.soft.eps;
        o.theta = sp.mac.theta;
        o.mac = sp.mac.kind == ngrav::MacKind::Relative ? NGRAV_MAC_RELATIVE : NGRAV_MAC_GEOMETRIC;
    }
    void Check(int rc) const {
        if (rc != NGRAV_OK) throw std::runtime_error(ngrav_gpu_last_error(m_ctx.get()));
    }

    std::shared_ptr<ngrav_gpu_ctx> m_ctx;
    std::shared_ptr<std::vector<double>> m_mass = std::make_shared<std::vector<double>>();  // last set's masses
    ngrav_gpu_opts m_opts{};
};

}  // namespace ngrav_gpu
