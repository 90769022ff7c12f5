// pbf_dual.cpp — dual-number (forward-mode) derivatives of the FP64 oracle
// twin (TEST INFRASTRUCTURE ONLY: used by tests/ to check the adjoint).
#include <vector>

#include "pbf_oracle.hpp"
#include "pbf_dual.hpp"

namespace {

constexpr int kLanes = 16;

template <typename V>
int dual_tangents(const pbfo::Params* prm, uint32_t n, const float* x4, const float* v4,
                  uint32_t substeps, uint32_t ndir, const int32_t* kind, const int32_t* idx,
                  const int32_t* comp, double* x_out, double* v_out, double* xdot, double* vdot,
                  int nthreads) {
    using D = pbfo::DualT<V, kLanes>;
    if (!prm || !x4 || !v4 || (ndir && (!kind || !idx || !comp))) return 1;
    for (uint32_t k = 0; k < ndir; ++k) {
        if (kind[k] < 0 || kind[k] > 5) return 1;
        if (kind[k] <= 1 && (idx[k] < 0 || (uint32_t)idx[k] >= n || comp[k] < 0 || comp[k] > 2))
            return 1;
    }
    const uint32_t passes = ndir ? (ndir + kLanes - 1) / kLanes : 1;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        pbfo::Sim<D> s;
        s.init(*prm, n);
        s.nthreads = nthreads;
        for (uint32_t i = 0; i < n; ++i) {
            s.x[i] = {D(x4[4 * i]), D(x4[4 * i + 1]), D(x4[4 * i + 2])};
            s.v[i] = {D(v4[4 * i]), D(v4[4 * i + 1]), D(v4[4 * i + 2])};
        }
        const uint32_t k0 = pass * kLanes;
        for (uint32_t k = k0; k < ndir && k < k0 + kLanes; ++k) {
            const int lane = (int)(k - k0);
            auto comp_of = [&](pbfo::V3<D>& a) -> D& { return comp[k] == 0 ? a.x : comp[k] == 1 ? a.y : a.z; };
            switch (kind[k]) {
                case 0: comp_of(s.v[idx[k]]).d[lane] = 1.0; break;
                case 1: comp_of(s.x[idx[k]]).d[lane] = 1.0; break;
                case 2: s.c.eps.d[lane] = 1.0; break;
                case 3: s.c.negk.d[lane] = -1.0; break;  // negk = -k
                case 4: s.c.cx.d[lane] = 1.0; break;
                case 5: s.c.dteps.d[lane] = (double)(V)prm->timestep; break;  // dteps = dt * eps_v
            }
        }
        for (uint32_t t = 0; t < substeps; ++t) s.substep();
        if (pass == 0) {
            for (uint32_t i = 0; i < n; ++i) {
                if (x_out) {
                    x_out[3 * i] = (double)s.x[i].x.v;
                    x_out[3 * i + 1] = (double)s.x[i].y.v;
                    x_out[3 * i + 2] = (double)s.x[i].z.v;
                }
                if (v_out) {
                    v_out[3 * i] = (double)s.v[i].x.v;
                    v_out[3 * i + 1] = (double)s.v[i].y.v;
                    v_out[3 * i + 2] = (double)s.v[i].z.v;
                }
            }
        }
        for (uint32_t k = k0; k < ndir && k < k0 + kLanes; ++k) {
            const int lane = (int)(k - k0);
            const size_t base = (size_t)k * n * 3;
            for (uint32_t i = 0; i < n; ++i) {
                if (xdot) {
                    xdot[base + 3 * i] = s.x[i].x.d[lane];
                    xdot[base + 3 * i + 1] = s.x[i].y.d[lane];
                    xdot[base + 3 * i + 2] = s.x[i].z.d[lane];
                }
                if (vdot) {
                    vdot[base + 3 * i] = s.v[i].x.d[lane];
                    vdot[base + 3 * i + 1] = s.v[i].y.d[lane];
                    vdot[base + 3 * i + 2] = s.v[i].z.d[lane];
                }
            }
        }
    }
    return 0;
}

}  // namespace

extern "C" {

// Tangents of the final state of `substeps` substeps along `ndir` directions.
// Direction k seeds kind[k]: 0 = v0[idx[k]][comp[k]], 1 = x0[idx[k]][comp[k]],
// 2 = epsilon, 3 = s_corr k (tensile_instability_k), 4 = XSPH c,
// 5 = vorticity epsilon.  Outputs (any may be NULL): x_out, v_out[n * 3]
// (the final state's value, equal to the FP64 twin's), xdot, vdot[ndir * n * 3]
// (d final state / d direction).  Runs ceil(ndir / 16) passes of the dual
// simulation.  Returns 0, or 1 on a bad argument.
int pbfo_dual_tangents(const pbfo::Params* prm, uint32_t n, const float* x4, const float* v4,
                       uint32_t substeps, uint32_t ndir, const int32_t* kind, const int32_t* idx,
                       const int32_t* comp, double* x_out, double* v_out, double* xdot,
                       double* vdot, int nthreads) {
    return dual_tangents<double>(prm, n, x4, v4, substeps, ndir, kind, idx, comp, x_out, v_out,
                                 xdot, vdot, nthreads);
}

// The same on the FP32 oracle's trajectory: the value part equals the FP32
// oracle (and so the GPU) bit for bit; the tangents are the derivatives of
// that FP32 program, carried in double.
int pbfo_dual_tangents_fp32(const pbfo::Params* prm, uint32_t n, const float* x4, const float* v4,
                            uint32_t substeps, uint32_t ndir, const int32_t* kind,
                            const int32_t* idx, const int32_t* comp, double* x_out,
                            double* v_out, double* xdot, double* vdot, int nthreads) {
    return dual_tangents<float>(prm, n, x4, v4, substeps, ndir, kind, idx, comp, x_out, v_out,
                                xdot, vdot, nthreads);
}

}  // extern "C"
