/*
 * The reference's own OpenCL kernel sources, compiled unmodified as C++
 * through clshim.hpp, exposed as an oracle_kernels table. Built by
 * oracle/Makefile into oracle/_ref/libufoir_ref.so, only where the reference
 * tree is present (UFO_IR_REF points at its src/kernels directory). Nothing
 * from the reference is copied into this repository: the .cl files are
 * #included from that directory at compile time.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h). Each table entry runs one
 * NDRange with the global size the reference's host code uses, work-items
 * spread over OpenMP threads (every kernel here is per-work-item independent).
 */
#include <cstring>

#include "clshim.hpp"
#include "oracle.h"

namespace clshim {
thread_local size_t gid[3];
thread_local size_t gsize[3];
}

namespace ref_joseph {
#include "projector-parallel-joseph.cl"
}
namespace ref_ops {
#include "ufo-ir-basic-ops.cl"
}
namespace ref_tv {
#include "ufo-math-tvstd-method.cl"
}
namespace ref_grad {
#include "ufo-ir-gradient-processor.cl"
}

template <typename F>
static void ndrange2(size_t gx, size_t gy, F f)
{
#pragma omp parallel for collapse(2) schedule(dynamic, 256)
    for (size_t y = 0; y < gy; y++) {
        for (size_t x = 0; x < gx; x++) {
            clshim::gid[0] = x;
            clshim::gid[1] = y;
            clshim::gid[2] = 0;
            clshim::gsize[0] = gx;
            clshim::gsize[1] = gy;
            clshim::gsize[2] = 1;
            f();
        }
    }
}

static image2d_t im(oracle_image a)
{
    image2d_t r;
    r.data = a.data;
    r.width = a.width;
    r.height = a.height;
    return r;
}

/* subset_fp_real (…parallel-projector-task.c:563-625): NDRange (sino dims[0], subset.n). */
static void ref_fp(oracle_image vol, oracle_image sino, const float *sin_val, const float *cos_val,
                   oracle_dims dims, float axis_pos, oracle_subset part, float correction_scale)
{
    ref_joseph::UfoGeometryDims d;
    d.height = dims.height;
    d.width = dims.width;
    d.n_dets = dims.n_dets;
    d.n_angles = dims.n_angles;
    ref_joseph::UfoProjectionsSubset p;
    p.offset = part.offset;
    p.n = part.n;
    p.direction = part.direction ? ref_joseph::Vertical : ref_joseph::Horizontal;
    const image2d_t v = im(vol), s = im(sino);
    if (part.direction)
        ndrange2((size_t) sino.width, part.n, [&] {
            ref_joseph::FP_vert(v, s, s, sin_val, cos_val, d, axis_pos, p, correction_scale);
        });
    else
        ndrange2((size_t) sino.width, part.n, [&] {
            ref_joseph::FP_hor(v, s, s, sin_val, cos_val, d, axis_pos, p, correction_scale);
        });
}

/* subset_bp_real (…parallel-projector-task.c:501-560): NDRange = volume dims. */
static void ref_bp(oracle_image vol, oracle_image sino, float relax, const float *sin_val,
                   const float *cos_val, oracle_dims dims, float axis_pos, oracle_subset part)
{
    ref_joseph::UfoGeometryDims d;
    d.height = dims.height;
    d.width = dims.width;
    d.n_dets = dims.n_dets;
    d.n_angles = dims.n_angles;
    ref_joseph::UfoProjectionsSubset p;
    p.offset = part.offset;
    p.n = part.n;
    p.direction = part.direction ? ref_joseph::Vertical : ref_joseph::Horizontal;
    const image2d_t v = im(vol), s = im(sino);
    ndrange2((size_t) vol.width, (size_t) vol.height, [&] {
        ref_joseph::BP(v, v, s, relax, sin_val, cos_val, d, axis_pos, p);
    });
}

static void ref_set(oracle_image a, float value)
{
    const image2d_t o = im(a);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_set(o, value); });
}

static void ref_inv(oracle_image a)
{
    const image2d_t o = im(a);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_inv(o, o); });
}

static void ref_mul(oracle_image a, oracle_image b, oracle_image out)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_mul(x, y, o); });
}

static void ref_add(oracle_image a, oracle_image b, oracle_image out)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_add(x, y, o); });
}

static void ref_deduction(oracle_image a, oracle_image b, oracle_image out)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_deduction(x, y, o); });
}

static void ref_deduction2(oracle_image a, oracle_image b, float m, oracle_image out)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_deduction2(x, y, m, o); });
}

static void ref_add2(oracle_image a, oracle_image b, float m, oracle_image out)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::operation_add2(x, y, m, o); });
}

/* ufo_ir_op_mul_rows (src/core/ufo-ir-basic-ops.c:206-251): NDRange (dims[0], n). */
static void ref_mul_rows(oracle_image a, oracle_image b, oracle_image out, unsigned int offset,
                         unsigned int n)
{
    const image2d_t x = im(a), y = im(b), o = im(out);
    ndrange2((size_t) out.width, n, [&] { ref_ops::op_mulRows(x, y, o, offset); });
}

static void ref_posc(oracle_image a, oracle_image out)
{
    const image2d_t x = im(a), o = im(out);
    ndrange2((size_t) a.width, (size_t) a.height, [&] { ref_ops::POSC(x, o); });
}

static void ref_l1_grad(oracle_image in, oracle_image out)
{
    const image2d_t x = im(in), o = im(out);
    ndrange2((size_t) in.width, (size_t) in.height, [&] { ref_tv::l1_grad(x, o); });
}

/* Gradient processor (src/core/ufo-ir-gradient-processor.c:74-155). */
static void ref_dx(const float *in, float *out, long w, long h)
{
    ndrange2((size_t) w, (size_t) h, [&] { ref_grad::Dx((float *) in, out); });
}

static void ref_dxt(const float *in, float *out, long w, long h)
{
    const int stop = (int) w - 1;
    ndrange2((size_t) w, (size_t) h, [&] { ref_grad::Dxt((float *) in, stop, out); });
}

static void ref_dy(const float *in, float *out, long w, long h)
{
    const int last = (int) (w * h);
    ndrange2((size_t) w, (size_t) h, [&] { ref_grad::Dy((float *) in, last, out); });
}

static void ref_dyt(const float *in, float *out, long w, long h)
{
    const int last = (int) (w * h), stop = (int) h - 1;
    ndrange2((size_t) w, (size_t) h, [&] { ref_grad::Dyt((float *) in, last, stop, out); });
}

static const oracle_kernels ref_table = {
    ref_fp, ref_bp, ref_set, ref_inv, ref_mul, ref_add, ref_deduction, ref_deduction2,
    ref_add2, ref_mul_rows, ref_posc, ref_l1_grad, ref_dx, ref_dxt, ref_dy, ref_dyt,
};

extern "C" const oracle_kernels *oracle_ref_kernels(void)
{
    return &ref_table;
}
