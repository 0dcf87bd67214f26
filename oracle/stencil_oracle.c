/*
 * stencil_oracle.c — CPU restatement of Stencils.jl's gatherstencil / mapstencil path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for libstencilcuda.so: the parity tests,
 * `__graft_entry__.smoke()` and the `cpu_baseline` / `--impl reference` legs of bench.py load it;
 * nothing in the product links or calls it.
 *
 * It follows the reference (Stencils.jl v0.3.6) step by step, on host memory, for every logical
 * index I in column-major order:
 *   gatherstencil!(f, dest, source)          src/gatherstencil.jl:89-103, :105-109
 *     update_boundary!(source)               src/array.jl:195-233 (halo_val :235-239)
 *     dest[I] = f(stencil(source, I))        src/array.jl:22-30
 *       unsafe_neighbors (Halo: parent[J+R]) src/array.jl:94-100, :347-349, :367-377
 *       unsafe_neighbors (Conditional: corner check, then fast or checked path)  src/array.jl:101-115
 *       getneighbor (Remove -> padval)       src/array.jl:133-135
 *       getneighbor (Wrap/Reflect)           src/array.jl:137-138, bounded_index :154-179
 *       _center                              src/array.jl:32
 *   gatherstencil!(f, ::SwitchingStencilArray) + switch   src/gatherstencil.jl:77-83, src/array.jl:610-611
 * The reductions fold left to right over the neighbours in offset order, as StaticArrays'
 * unrolled `_mapfoldl` does for `sum`/`mean`/`minimum`/`maximum` (first element taken as is,
 * `Base.reduce_first`), and as `kernelproduct` (src/stencils/kernel.jl:37-43) does from zero.
 * StaticArrays.jl and Statistics.jl (compat "1", Project.toml:29-30) are not vendored and no
 * Manifest pins their versions; the fold order above is their published algorithm.
 *
 * Floating point is evaluated without contraction (build with -ffp-contract=off): Julia does
 * not fuse `s += a * b` unless asked to.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/stencil_cuda.h"

/* ---------------------------------------------------------------- element access */

static int is_float_dtype(int dt) { return dt == STC_F64 || dt == STC_F32 || dt == STC_BF16 || dt == STC_F16; }

static size_t dtype_size(int dt) {
    switch (dt) {
    case STC_F64: case STC_I64: return 8;
    case STC_F32: case STC_I32: return 4;
    case STC_BF16: case STC_F16: return 2;
    case STC_U8: case STC_BOOL: return 1;
    default: return 0;
    }
}

static float bf16_to_f32(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* round-to-nearest-even float -> bfloat16, NaN kept quiet */
static uint16_t f32_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x0040u);
    uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    return (uint16_t)(u >> 16);
}

static double load_f(const void* base, int dt, int64_t off) {
    switch (dt) {
    case STC_F64: return ((const double*)base)[off];
    case STC_F32: return (double)((const float*)base)[off];
    case STC_BF16: return (double)bf16_to_f32(((const uint16_t*)base)[off]);
    case STC_F16: return (double)((const _Float16*)base)[off];
    case STC_U8: case STC_BOOL: return (double)((const uint8_t*)base)[off];
    case STC_I32: return (double)((const int32_t*)base)[off];
    case STC_I64: return (double)((const int64_t*)base)[off];
    }
    return 0.0;
}

static int64_t load_i(const void* base, int dt, int64_t off) {
    switch (dt) {
    case STC_U8: case STC_BOOL: return ((const uint8_t*)base)[off];
    case STC_I32: return ((const int32_t*)base)[off];
    case STC_I64: return ((const int64_t*)base)[off];
    default: return (int64_t)load_f(base, dt, off);
    }
}

static void store_raw(void* base, int dt, int64_t off, const void* src) {
    memcpy((char*)base + off * (int64_t)dtype_size(dt), src, dtype_size(dt));
}

/* ---------------------------------------------------------------- descriptors */

typedef struct {
    int nd;                 /* grid dims */
    int64_t n[3];           /* logical size (1 beyond nd) */
    int64_t st[3];          /* parent strides */
    int64_t org;            /* parent offset of logical index 0 */
    int halo;               /* 1 for Halo padding */
    int R;
    int dt;
    const void* data;
} view_t;

static int make_view(const stc_grid* g, int R, int padding, view_t* v) {
    if (!g || !g->data || g->ndims < 1 || g->ndims > 3) return STC_ERR_INVALID;
    v->nd = g->ndims;
    v->halo = padding != STC_CONDITIONAL;
    v->R = R;
    v->dt = g->dtype;
    v->data = g->data;
    v->org = 0;
    for (int d = 0; d < 3; ++d) {
        if (d < g->ndims) {
            v->n[d] = g->size[d] - (v->halo ? 2 * R : 0);
            v->st[d] = g->stride[d];
            if (v->halo) v->org += (int64_t)R * g->stride[d];
        } else {
            v->n[d] = 1;
            v->st[d] = 0;
        }
    }
    /* StencilArray constructor check: radius < axis, on the parent (src/array.jl:451-453) */
    for (int d = 0; d < g->ndims; ++d)
        if (!(R < g->size[d])) return STC_ERR_RADIUS;
    for (int d = 0; d < g->ndims; ++d)
        if (v->n[d] < 0) return STC_ERR_RADIUS;
    return STC_OK;
}

/* parent offset of logical index J (0-based, may lie in the halo ring for Halo padding) */
static int64_t poff(const view_t* v, const int64_t J[3]) {
    return v->org + J[0] * v->st[0] + J[1] * v->st[1] + J[2] * v->st[2];
}

/* bounded_index for Wrap / Reflect, one axis, 0-based (src/array.jl:154-179) */
static int64_t bound_axis(int boundary, int64_t i, int64_t s) {
    if (boundary == STC_WRAP) {
        if (i < 0) return i + s;
        if (i >= s) return i - s;
        return i;
    }
    /* Reflect, 1-based: i<1 -> 2-i ; i>s -> 2s-i.  0-based j=i-1: j<0 -> -j ; j>=s -> 2s-2-j */
    if (i < 0) return -i;
    if (i >= s) return 2 * s - 2 - i;
    return i;
}

typedef union { double f; int64_t i; } val_t;

typedef struct {
    view_t src;
    const stc_stencil* st;
    const stc_bc* bc;
    int fkind;              /* 1: values gathered as double, 0: as int64 */
    double padf;            /* Remove's padval as a value of the source element type */
    int64_t padi;
} gather_t;

/* stencil(source, I): neighbours in offset order, plus the centre */
static void gather(const gather_t* g, const int64_t I[3], val_t* vals, val_t* centre) {
    const view_t* v = &g->src;
    const stc_stencil* st = g->st;
    const int L = st->len, sn = st->ndims;
    int64_t J[3];
    if (v->halo) {
        /* Halo: unsafe_getindex(A, Halo, J) = parent[J .+ R] — no boundary logic */
        for (int k = 0; k < L; ++k) {
            for (int d = 0; d < 3; ++d) J[d] = I[d] + (d < sn ? st->offsets[k * sn + d] : 0);
            int64_t o = poff(v, J);
            if (g->fkind) vals[k].f = load_f(v->data, v->dt, o); else vals[k].i = load_i(v->data, v->dt, o);
        }
    } else {
        /* Conditional: both corners I±R in bounds over all array dims -> unchecked reads */
        int fast = 1;
        for (int d = 0; d < v->nd; ++d)
            if (I[d] - v->R < 0 || I[d] + v->R >= v->n[d]) fast = 0;
        for (int k = 0; k < L; ++k) {
            for (int d = 0; d < 3; ++d) J[d] = I[d] + (d < sn ? st->offsets[k * sn + d] : 0);
            int inb = 1;
            for (int d = 0; d < v->nd; ++d)
                if (J[d] < 0 || J[d] >= v->n[d]) inb = 0;
            if (fast || inb) {
                int64_t o = poff(v, J);
                if (g->fkind) vals[k].f = load_f(v->data, v->dt, o); else vals[k].i = load_i(v->data, v->dt, o);
            } else if (g->bc->boundary == STC_REMOVE) {
                if (g->fkind) vals[k].f = g->padf; else vals[k].i = g->padi;
            } else {
                for (int d = 0; d < v->nd; ++d) J[d] = bound_axis(g->bc->boundary, J[d], v->n[d]);
                int64_t o = poff(v, J);
                if (g->fkind) vals[k].f = load_f(v->data, v->dt, o); else vals[k].i = load_i(v->data, v->dt, o);
            }
        }
    }
    int64_t o = poff(v, I);
    if (g->fkind) centre->f = load_f(v->data, v->dt, o); else centre->i = load_i(v->data, v->dt, o);
}

/* ---------------------------------------------------------------- type rules */

/* accumulation type: F64, F32, or an integer code meaning "int64 wrapped to dtype width" */
static int acc_dtype(int op, int sdt, int wdt) {
    int sf = is_float_dtype(sdt);
    switch (op) {
    case STC_OP_MEAN:
    case STC_OP_DIFFUSE:
        if (!sf) return op == STC_OP_MEAN ? STC_F64 : -1;
        return sdt == STC_F64 ? STC_F64 : STC_F32;
    case STC_OP_SUM:
        if (!sf) return sdt == STC_BOOL ? STC_I64 : sdt;
        return sdt == STC_F64 ? STC_F64 : STC_F32;
    case STC_OP_KDOT:
        if (!sf || sdt == STC_F64 || wdt == STC_F64) return STC_F64;
        return STC_F32;
    case STC_OP_MIN:
    case STC_OP_MAX:
        return sf ? (sdt == STC_F64 ? STC_F64 : STC_F32) : sdt;
    case STC_OP_LIFE:
        return sf ? -1 : STC_I64;
    }
    return -1;
}

int orc_result_dtype(int op, int sdt, int wdt) {
    int a = acc_dtype(op, sdt, wdt);
    if (a < 0) return STC_ERR_UNSUPPORTED;
    switch (op) {
    case STC_OP_MEAN:
        return is_float_dtype(sdt) ? sdt : STC_F64;
    case STC_OP_SUM:
        return is_float_dtype(sdt) ? sdt : a;
    case STC_OP_KDOT:
        if (is_float_dtype(sdt) && sdt != STC_F64 && a == STC_F32) return sdt;
        return STC_F64;
    case STC_OP_MIN: case STC_OP_MAX: case STC_OP_LIFE: case STC_OP_DIFFUSE:
        return sdt;
    }
    return STC_ERR_UNSUPPORTED;
}

static int64_t wrap_int(int64_t x, int dt) {
    switch (dt) {
    case STC_U8: case STC_BOOL: return (int64_t)(uint8_t)x;
    case STC_I32: return (int64_t)(int32_t)(uint32_t)(uint64_t)x;
    default: return x;
    }
}

/* Julia's min/max on floats: NaN-propagating, -0.0 < +0.0 */
static double jl_min(double x, double y) {
    if (isnan(x) || isnan(y)) return NAN;
    return (x < y || (x == y && signbit(x))) ? x : y;
}
static double jl_max(double x, double y) {
    if (isnan(x) || isnan(y)) return NAN;
    return (x > y || (x == y && !signbit(x))) ? x : y;
}
static float jl_minf(float x, float y) {
    if (isnan(x) || isnan(y)) return NAN;
    return (x < y || (x == y && signbit(x))) ? x : y;
}
static float jl_maxf(float x, float y) {
    if (isnan(x) || isnan(y)) return NAN;
    return (x > y || (x == y && !signbit(x))) ? x : y;
}

/* store an f64- or f32-accumulated result into a float dst */
static void store_float(void* base, int dt, int64_t off, double x64, float x32, int acc) {
    switch (dt) {
    case STC_F64: { double v = acc == STC_F64 ? x64 : (double)x32; store_raw(base, dt, off, &v); break; }
    case STC_F32: { float v = acc == STC_F64 ? (float)x64 : x32; store_raw(base, dt, off, &v); break; }
    case STC_BF16: { uint16_t v = f32_to_bf16(acc == STC_F64 ? (float)x64 : x32); store_raw(base, dt, off, &v); break; }
    case STC_F16: { _Float16 v = acc == STC_F64 ? (_Float16)x64 : (_Float16)x32; store_raw(base, dt, off, &v); break; }
    }
}

static void store_int(void* base, int dt, int64_t off, int64_t x) {
    switch (dt) {
    case STC_U8: case STC_BOOL: { uint8_t v = (uint8_t)x; store_raw(base, dt, off, &v); break; }
    case STC_I32: { int32_t v = (int32_t)(uint32_t)(uint64_t)x; store_raw(base, dt, off, &v); break; }
    case STC_I64: { store_raw(base, dt, off, &x); break; }
    }
}

/* f(hood) for one cell; writes dst */
static void reduce_store(const stc_op* op, const stc_stencil* st, int acc, int sdt,
                         const val_t* vals, val_t centre, void* dbase, int ddt, int64_t doff) {
    const int L = st->len;
    switch (op->code) {
    case STC_OP_MEAN:
    case STC_OP_SUM:
    case STC_OP_DIFFUSE:
        if (acc == STC_F64) {
            double s = vals[0].f;
            for (int k = 1; k < L; ++k) s = s + vals[k].f;
            if (op->code == STC_OP_MEAN) s = s / (double)L;
            if (op->code == STC_OP_DIFFUSE) {
                double c = centre.f;
                double t = (double)L * c;
                t = s - t;
                t = op->alpha * t;
                s = c + t;
            }
            store_float(dbase, ddt, doff, s, 0.f, acc);
        } else if (acc == STC_F32) {
            float s = (float)vals[0].f;
            for (int k = 1; k < L; ++k) s = s + (float)vals[k].f;
            if (op->code == STC_OP_MEAN) s = s / (float)L;
            if (op->code == STC_OP_DIFFUSE) {
                float c = (float)centre.f;
                float t = (float)L * c;
                t = s - t;
                t = (float)op->alpha * t;
                s = c + t;
            }
            store_float(dbase, ddt, doff, 0.0, s, acc);
        } else {
            /* integer sum: Bool widens to Int (reduce_first), others wrap at their width */
            int64_t s = vals[0].i;
            for (int k = 1; k < L; ++k) s = wrap_int((int64_t)((uint64_t)s + (uint64_t)vals[k].i), acc);
            store_int(dbase, ddt, doff, s);
        }
        break;
    case STC_OP_KDOT:
        if (acc == STC_F64) {
            double s = 0.0;
            for (int k = 0; k < L; ++k) {
                double p = vals[k].f * st->weights[k];
                s = s + p;
            }
            store_float(dbase, ddt, doff, s, 0.f, acc);
        } else {
            float s = 0.0f;
            for (int k = 0; k < L; ++k) {
                float p = (float)vals[k].f * (float)st->weights[k];
                s = s + p;
            }
            store_float(dbase, ddt, doff, 0.0, s, acc);
        }
        break;
    case STC_OP_MIN:
    case STC_OP_MAX: {
        int mx = op->code == STC_OP_MAX;
        if (acc == STC_F64) {
            double s = vals[0].f;
            for (int k = 1; k < L; ++k) s = mx ? jl_max(s, vals[k].f) : jl_min(s, vals[k].f);
            store_float(dbase, ddt, doff, s, 0.f, acc);
        } else if (acc == STC_F32) {
            float s = (float)vals[0].f;
            for (int k = 1; k < L; ++k) s = mx ? jl_maxf(s, (float)vals[k].f) : jl_minf(s, (float)vals[k].f);
            store_float(dbase, ddt, doff, 0.0, s, acc);
        } else {
            int64_t s = vals[0].i;
            for (int k = 1; k < L; ++k) s = mx ? (vals[k].i > s ? vals[k].i : s) : (vals[k].i < s ? vals[k].i : s);
            store_int(dbase, ddt, doff, s);
        }
        break;
    }
    case STC_OP_LIFE: {
        int n = 0;
        for (int k = 0; k < L; ++k) n += vals[k].i != 0;
        uint32_t mask = centre.i != 0 ? op->survive_mask : op->birth_mask;
        store_int(dbase, ddt, doff, (int64_t)((mask >> n) & 1u));
        break;
    }
    }
    (void)sdt;
}

/* ---------------------------------------------------------------- validation */

static int check_args(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st,
                      const stc_op* op, const stc_bc* bc) {
    if (!src || !dst || !st || !op || !bc || !st->offsets) return STC_ERR_INVALID;
    if (st->len < 1 || st->len > STC_MAX_LEN || st->ndims < 1 || st->ndims > src->ndims) return STC_ERR_INVALID;
    if (src->stride[0] != 1 || dst->stride[0] != 1) return STC_ERR_INVALID;
    for (int k = 0; k < st->len * st->ndims; ++k)
        if (abs(st->offsets[k]) > st->radius) return STC_ERR_UNSUPPORTED;
    if (op->code == STC_OP_KDOT && !st->weights) return STC_ERR_KERNEL_LENGTH;
    if (op->code == STC_OP_LIFE && st->len > 31) return STC_ERR_UNSUPPORTED;
    if (bc->boundary == STC_USE && bc->padding == STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    if (acc_dtype(op->code, src->dtype, st->weight_dtype) < 0) return STC_ERR_UNSUPPORTED;
    if (dst->ndims != src->ndims) return STC_ERR_SIZE_MISMATCH;
    int halo = bc->padding != STC_CONDITIONAL;
    for (int d = 0; d < src->ndims; ++d) {
        int64_t logical = src->size[d] - (halo ? 2 * st->radius : 0);
        int64_t want = logical + ((halo && dst_padded) ? 2 * st->radius : 0);
        if (dst->size[d] != want) return STC_ERR_SIZE_MISMATCH;
    }
    int acc = acc_dtype(op->code, src->dtype, st->weight_dtype);
    int acc_f = acc == STC_F64 || acc == STC_F32;
    if (acc_f != is_float_dtype(dst->dtype)) return STC_ERR_UNSUPPORTED;
    return STC_OK;
}

/* ---------------------------------------------------------------- update_boundary! */

int orc_update_boundary(const stc_grid* parent, int R, const stc_bc* bc) {
    if (bc->padding == STC_CONDITIONAL || bc->boundary == STC_USE) return STC_OK;  /* src/array.jl:199-200 */
    view_t v;
    int rc = make_view(parent, R, bc->padding, &v);
    if (rc) return rc;
    int fk = is_float_dtype(v.dt);
    void* base = (void*)v.data;
    /* slab per dimension i: indices 1:R and s+R+1:s+2R along i, full padded extent elsewhere */
    for (int i = 0; i < v.nd; ++i) {
        int64_t lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = d < v.nd ? -R : 0;
            hi[d] = d < v.nd ? v.n[d] + R : 1;
        }
        for (int side = 0; side < 2; ++side) {
            int64_t a0 = side == 0 ? -R : v.n[i];
            int64_t a1 = side == 0 ? 0 : v.n[i] + R;
            int64_t L0[3] = {lo[0], lo[1], lo[2]}, L1[3] = {hi[0], hi[1], hi[2]};
            L0[i] = a0;
            L1[i] = a1;
            int64_t J[3];
            for (J[2] = L0[2]; J[2] < L1[2]; ++J[2])
                for (J[1] = L0[1]; J[1] < L1[1]; ++J[1])
                    for (J[0] = L0[0]; J[0] < L1[0]; ++J[0]) {
                        int64_t dsto = poff(&v, J);
                        if (bc->boundary == STC_REMOVE) {
                            if (fk) store_float(base, v.dt, dsto, bc->padval, (float)bc->padval, STC_F64);
                            else store_int(base, v.dt, dsto, bc->padval_int);
                        } else {
                            int64_t B[3];
                            for (int d = 0; d < 3; ++d)
                                B[d] = d < v.nd ? bound_axis(bc->boundary, J[d], v.n[d]) : J[d];
                            int64_t so = poff(&v, B);
                            store_raw(base, v.dt, dsto, (const char*)v.data + so * (int64_t)dtype_size(v.dt));
                        }
                    }
        }
    }
    return STC_OK;
}

/* ---------------------------------------------------------------- the map */

/* Specialised restatement for Moore(1) outer-totalistic rules on UInt8 / Bool Halo parents: what the
 * reference's compiled kernel does for that stencil type (compile-time offsets, neighbours read straight
 * from the padded parent, src/array.jl:347-349), so the CPU baseline is not a generic interpreter.
 * Integer counts, so the result equals the generic gather's bit for bit (tested). */
static int g_fast_paths = 1;
void orc_set_fast_paths(int on) { g_fast_paths = on != 0; }

static int is_moore1_table(const stc_stencil* st) {
    if (st->ndims != 2 || st->len != 8 || st->radius != 1) return 0;
    int seen = 0;
    for (int k = 0; k < 8; ++k) {
        const int x = st->offsets[2 * k], y = st->offsets[2 * k + 1];
        if (x < -1 || x > 1 || y < -1 || y > 1 || (x == 0 && y == 0)) return 0;
        const int bit = 1 << ((y + 1) * 3 + (x + 1));
        if (seen & bit) return 0;
        seen |= bit;
    }
    return 1;
}

static int life_fast(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_op* op, int nthreads) {
    const int64_t n0 = src->size[0] - 2, n1 = src->size[1] - 2;
    const int64_t ps = src->stride[1], ds = dst->stride[1];
    const uint8_t* P = (const uint8_t*)src->data;
    uint8_t* D = (uint8_t*)dst->data + (dst_padded ? 1 + ds : 0);
    /* next state = bit n of the survive (alive) or birth (dead) mask, n = live neighbours (0..8): formed
     * as nine compare / select steps on 8-bit lanes so the row loop vectorises */
    uint8_t bm[9], sm[9];
    for (int v = 0; v < 9; ++v) {
        bm[v] = (uint8_t)((op->birth_mask >> v) & 1u);
        sm[v] = (uint8_t)((op->survive_mask >> v) & 1u);
    }
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t j = 0; j < n1; ++j) {
        const uint8_t* up = P + j * ps;     /* parent row of logical j - 1 */
        const uint8_t* mid = up + ps;
        const uint8_t* dn = mid + ps;
        uint8_t* out = D + j * ds;
        for (int64_t i = 0; i < n0; ++i) {
            const uint8_t n = (uint8_t)((up[i] != 0) + (up[i + 1] != 0) + (up[i + 2] != 0) + (mid[i] != 0) +
                                        (mid[i + 2] != 0) + (dn[i] != 0) + (dn[i + 1] != 0) + (dn[i + 2] != 0));
            const uint8_t alive = mid[i + 1] != 0;
            uint8_t o = 0;
#pragma GCC unroll 9
            for (int v = 0; v < 9; ++v) o |= (uint8_t)((n == v) & (alive ? sm[v] : bm[v]));
            out[i] = o;
        }
    }
    return STC_OK;
}

int orc_map(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st,
            const stc_op* op, const stc_bc* bc, int nthreads) {
    int rc = check_args(src, dst, dst_padded, st, op, bc);
    if (rc) return rc;
    rc = orc_update_boundary(src, st->radius, bc);
    if (rc) return rc;
    if (g_fast_paths && op->code == STC_OP_LIFE && src->ndims == 2 && src->dtype == dst->dtype &&
        (src->dtype == STC_U8 || src->dtype == STC_BOOL) && bc->padding != STC_CONDITIONAL &&
        is_moore1_table(st) && src->stride[0] == 1 && (dst->size[0] <= 1 || dst->stride[0] == 1))
        return life_fast(src, dst, dst_padded, op, nthreads);
    gather_t g;
    rc = make_view(src, st->radius, bc->padding, &g.src);
    if (rc) return rc;
    g.st = st;
    g.bc = bc;
    int acc = acc_dtype(op->code, src->dtype, st->weight_dtype);
    g.fkind = is_float_dtype(src->dtype) || acc == STC_F64 || acc == STC_F32;
    if (op->code == STC_OP_LIFE) g.fkind = 0;
    g.padi = wrap_int(bc->padval_int, src->dtype);
    switch (src->dtype) {
    case STC_F64: g.padf = bc->padval; break;
    case STC_F32: g.padf = (double)(float)bc->padval; break;
    case STC_BF16: g.padf = (double)bf16_to_f32(f32_to_bf16((float)bc->padval)); break;
    case STC_F16: g.padf = (double)(_Float16)bc->padval; break;
    default: g.padf = (double)g.padi; break;
    }
    const int64_t n0 = g.src.n[0], n1 = g.src.n[1], n2 = g.src.n[2];
    const int64_t total = n0 * n1 * n2;
    int64_t dorg = 0;
    int halo = bc->padding != STC_CONDITIONAL;
    if (halo && dst_padded)
        for (int d = 0; d < dst->ndims; ++d) dorg += (int64_t)st->radius * dst->stride[d];
    int64_t dst_st[3] = {dst->stride[0], dst->ndims > 1 ? dst->stride[1] : 0, dst->ndims > 2 ? dst->stride[2] : 0};
    if (nthreads < 1) nthreads = 1;
    /* Float64 / Float32 sum and mean: cells whose whole stencil lies inside the parent's valid data
     * (every cell under Halo padding; the interior under Conditional, the reference's unchecked corner
     * path, src/array.jl:104-114) fold straight from the parent through constant linear offsets, in
     * table order and the same arithmetic as the generic gather; the other cells take the gather. */
    const int ffast = g_fast_paths && (op->code == STC_OP_MEAN || op->code == STC_OP_SUM) &&
                      acc == src->dtype && dst->dtype == src->dtype &&
                      (src->dtype == STC_F64 || src->dtype == STC_F32) && st->len <= STC_MAX_LEN;
    int64_t lo[3] = {0, 0, 0}, hi[3] = {n0, n1, n2};
    int64_t* loff = NULL;
    if (ffast) {
        loff = (int64_t*)malloc(sizeof(int64_t) * (size_t)st->len);
        for (int k = 0; k < st->len; ++k) {
            loff[k] = 0;
            for (int d = 0; d < st->ndims; ++d) loff[k] += (int64_t)st->offsets[k * st->ndims + d] * g.src.st[d];
        }
        if (!halo)
            for (int d = 0; d < g.src.nd; ++d) {
                lo[d] = st->radius;
                hi[d] = g.src.n[d] - st->radius;
            }
    }
#pragma omp parallel num_threads(nthreads)
    {
        val_t* vals = (val_t*)malloc(sizeof(val_t) * (size_t)st->len);
#pragma omp for schedule(static)
        for (int64_t row = 0; row < n1 * n2; ++row) {
            const int64_t y = row % n1, z = row / n1;
            const int inner_row = ffast && y >= lo[1] && y < hi[1] && z >= lo[2] && z < hi[2];
            const int64_t xa = inner_row ? (lo[0] < n0 ? lo[0] : n0) : n0;
            const int64_t xb = inner_row ? (hi[0] > xa ? hi[0] : xa) : n0;
            for (int64_t x = 0; x < n0; ++x) {
                if (x == xa && xb > xa) {
                    const int64_t I0[3] = {xa, y, z};
                    const int64_t pb = poff(&g.src, I0);
                    const int64_t db = dorg + xa * dst_st[0] + y * dst_st[1] + z * dst_st[2];
                    const int L = st->len;
                    if (src->dtype == STC_F64) {
                        const double* sp = (const double*)g.src.data + pb;
                        double* dp = (double*)dst->data + db;
                        for (int64_t t = 0; t < xb - xa; ++t) {
                            double a = sp[t + loff[0]];
                            for (int k = 1; k < L; ++k) a = a + sp[t + loff[k]];
                            dp[t] = op->code == STC_OP_MEAN ? a / (double)L : a;
                        }
                    } else {
                        const float* sp = (const float*)g.src.data + pb;
                        float* dp = (float*)dst->data + db;
                        for (int64_t t = 0; t < xb - xa; ++t) {
                            float a = sp[t + loff[0]];
                            for (int k = 1; k < L; ++k) a = a + sp[t + loff[k]];
                            dp[t] = op->code == STC_OP_MEAN ? a / (float)L : a;
                        }
                    }
                    x = xb - 1;
                    continue;
                }
                int64_t I[3] = {x, y, z};
                val_t centre;
                gather(&g, I, vals, &centre);
                int64_t doff = dorg + I[0] * dst_st[0] + I[1] * dst_st[1] + I[2] * dst_st[2];
                reduce_store(op, st, acc, src->dtype, vals, centre, dst->data, dst->dtype, doff);
            }
        }
        free(vals);
    }
    free(loff);
    (void)total;
    return STC_OK;
}

/* nsteps of  A = mapstencil!(f, A)  on a SwitchingStencilArray with parents a (source) and b */
int orc_map_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                  const stc_bc* bc, int64_t nsteps, int nthreads, int* out_src_is_b) {
    const stc_grid* s = a;
    const stc_grid* d = b;
    for (int64_t k = 0; k < nsteps; ++k) {
        int rc = orc_map(s, d, 1, st, op, bc, nthreads);
        if (rc) return rc;
        const stc_grid* t = s;
        s = d;
        d = t;
    }
    if (out_src_is_b) *out_src_is_b = (s == b);
    return STC_OK;
}

/* Neumaier-compensated FP64 total over the logical grid */
double orc_mass(const stc_grid* g, int R, int padding) {
    view_t v;
    if (make_view(g, R, padding, &v)) return NAN;
    double s = 0.0, c = 0.0;
    int64_t J[3];
    for (J[2] = 0; J[2] < v.n[2]; ++J[2])
        for (J[1] = 0; J[1] < v.n[1]; ++J[1])
            for (J[0] = 0; J[0] < v.n[0]; ++J[0]) {
                double x = load_f(v.data, v.dt, poff(&v, J));
                double t = s + x;
                if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
                s = t;
            }
    return s + c;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

uint16_t orc_f32_to_bf16(float f) { return f32_to_bf16(f); }

/* ---------------------------------------------------------------- maps over several arrays */
/* mapstencil(f, A, args...) with f = t_1 + t_2 + ... (src/gatherstencil.jl:84-113): term m is
 * center(hood), sum / mean / kernelproduct of the neighbours of argument m's stencil at I, or the
 * value of a plain array at I (`_getarg`, src/gatherstencil.jl:111-112), optionally alpha * term.
 * Arithmetic in the element type T (Float64 or Float32), each operation rounded, left to right. */
#define ORC_TERM_BODY(T)                                                                               \
    do {                                                                                               \
        T acc = 0;                                                                                     \
        for (int m = 0; m < nterms; ++m) {                                                             \
            const stc_term* tm = &terms[m];                                                            \
            T g;                                                                                       \
            if (tm->kind == STC_TERM_VALUE) {                                                          \
                g = (T)load_f(vw[m].data, vw[m].dt, poff(&vw[m], I));                                  \
            } else {                                                                                   \
                val_t centre;                                                                          \
                gather(&gt[m], I, vals, &centre);                                                      \
                const int L = tm->stencil->len;                                                        \
                if (tm->kind == STC_TERM_CENTER) {                                                     \
                    g = (T)centre.f;                                                                   \
                } else if (tm->kind == STC_TERM_KDOT) {                                                \
                    g = (T)0;                                                                          \
                    for (int k = 0; k < L; ++k) {                                                      \
                        T w = (T)tm->stencil->weights[k];                                              \
                        T prod = (T)vals[k].f * w;                                                     \
                        g = g + prod;                                                                  \
                    }                                                                                  \
                } else {                                                                               \
                    g = (T)vals[0].f;                                                                  \
                    for (int k = 1; k < L; ++k) g = g + (T)vals[k].f;                                  \
                    if (tm->kind == STC_TERM_MEAN) g = g / (T)L;                                       \
                }                                                                                      \
            }                                                                                          \
            if (tm->scaled) g = (T)tm->alpha * g;                                                      \
            acc = m == 0 ? g : acc + g;                                                                \
        }                                                                                              \
        T out = acc;                                                                                   \
        store_raw(dst->data, dst->dtype, doff, &out);                                                  \
    } while (0)

int orc_map_terms(const stc_term* terms, int nterms, const stc_grid* dst, int dst_padded, int nthreads) {
    if (!terms || !dst || nterms < 1 || nterms > STC_MAX_TERMS) return STC_ERR_INVALID;
    const int dt = dst->dtype;
    if (dt != STC_F64 && dt != STC_F32) return STC_ERR_UNSUPPORTED;
    view_t vw[STC_MAX_TERMS];
    gather_t gt[STC_MAX_TERMS];
    int maxL = 1;
    for (int m = 0; m < nterms; ++m) {
        const stc_term* tm = &terms[m];
        if (!tm->grid || tm->grid->dtype != dt || tm->grid->ndims != dst->ndims) return STC_ERR_INVALID;
        if (tm->kind == STC_TERM_VALUE) {
            int rc = make_view(tm->grid, 0, STC_CONDITIONAL, &vw[m]);
            if (rc) return rc;
        } else {
            const stc_stencil* st = tm->stencil;
            const stc_bc* bc = tm->bc;
            if (!st || !bc) return STC_ERR_INVALID;
            if (bc->boundary == STC_USE && bc->padding == STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
            if (tm->kind == STC_TERM_KDOT && !st->weights) return STC_ERR_KERNEL_LENGTH;
            int rc = orc_update_boundary(tm->grid, st->radius, bc);
            if (rc) return rc;
            rc = make_view(tm->grid, st->radius, bc->padding, &gt[m].src);
            if (rc) return rc;
            vw[m] = gt[m].src;
            gt[m].st = st;
            gt[m].bc = bc;
            gt[m].fkind = 1;
            gt[m].padf = dt == STC_F32 ? (double)(float)bc->padval : bc->padval;
            gt[m].padi = 0;
            if (st->len > maxL) maxL = st->len;
        }
        for (int d = 0; d < 3; ++d)
            if (vw[m].n[d] != vw[0].n[d]) return STC_ERR_SIZE_MISMATCH;
    }
    const int R0 = (terms[0].kind != STC_TERM_VALUE && terms[0].bc->padding != STC_CONDITIONAL)
                       ? terms[0].stencil->radius : 0;
    int64_t dorg = 0;
    for (int d = 0; d < dst->ndims; ++d) {
        if (dst->size[d] != vw[0].n[d] + (dst_padded ? 2 * R0 : 0)) return STC_ERR_SIZE_MISMATCH;
        if (dst_padded) dorg += (int64_t)R0 * dst->stride[d];
    }
    const int64_t n0 = vw[0].n[0], n1 = vw[0].n[1], n2 = vw[0].n[2];
    const int64_t total = n0 * n1 * n2;
    int64_t dst_st[3] = {dst->stride[0], dst->ndims > 1 ? dst->stride[1] : 0, dst->ndims > 2 ? dst->stride[2] : 0};
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
    {
        val_t* vals = (val_t*)malloc(sizeof(val_t) * (size_t)maxL);
#pragma omp for schedule(static)
        for (int64_t lin = 0; lin < total; ++lin) {
            int64_t I[3] = {lin % n0, (lin / n0) % n1, lin / (n0 * n1)};
            int64_t doff = dorg + I[0] * dst_st[0] + I[1] * dst_st[1] + I[2] * dst_st[2];
            if (dt == STC_F64) ORC_TERM_BODY(double);
            else ORC_TERM_BODY(float);
        }
        free(vals);
    }
    return STC_OK;
}

/* ---------------------------------------------------------------- scatterstencil! */
/* scatterstencil!(f, op, dest, source) (src/scatterstencil.jl:36-74): passes over the columns
 * j = p, p + stride, ... (stride = 2R + 1), rows in order, offsets in order; targets mapped by
 * _scatter_to! (src/scatterstencil.jl:76-112): Remove/Use skip, Wrap mod1, Reflect 2 - i / 2n - i.
 * The columns of a pass may run on threads (orc_scatter below); every dest cell still receives its
 * contributions in the order of a one-thread run. */
static int scatter_target(int boundary, int64_t t, int64_t n, int64_t* out) {
    if (t >= 0 && t < n) { *out = t; return 1; }
    if (boundary == STC_WRAP) { int64_t m = t % n; *out = m < 0 ? m + n : m; return 1; }
    if (boundary == STC_REFLECT) { *out = t < 0 ? -t : 2 * n - 2 - t; return 1; }
    return 0;
}

#define ORC_SCATTER_BODY(T, ADDF, MAXF, MINF)                                                          \
    do {                                                                                               \
        T* d = (T*)dst->data;                                                                          \
        for (int64_t p = 0; p < stride; ++p) {                                                         \
            const int64_t ncol = p < nx ? (nx - p + stride - 1) / stride : 0;                          \
            _Pragma("omp parallel for num_threads(nt) schedule(static)")                               \
            for (int64_t cj = 0; cj < ncol; ++cj)                                                      \
                for (int64_t i = 0, j = p + cj * stride; i < ny; ++i) {                                \
                    const int64_t I[3] = {i, j, 0};                                                    \
                    const T c = (T)load_f(v.data, v.dt, poff(&v, I));                                  \
                    for (int k = 0; k < st->len; ++k) {                                                \
                        T val;                                                                         \
                        if (op->value == STC_SCATTER_CONST) val = (T)op->constant;                     \
                        else if (op->value == STC_SCATTER_CENTER) val = c;                             \
                        else { T w = (T)st->weights[k]; val = c * w; }                                 \
                        int64_t ti, tj;                                                                \
                        if (!scatter_target(bc->boundary, i + st->offsets[2 * k], ny, &ti)) continue;  \
                        if (!scatter_target(bc->boundary, j + st->offsets[2 * k + 1], nx, &tj)) continue; \
                        T* q = d + ti * dst->stride[0] + tj * dst->stride[1];                          \
                        if (op->combine == STC_COMBINE_ADD) *q = ADDF(*q, val);                        \
                        else if (op->combine == STC_COMBINE_MAX) *q = MAXF(*q, val);                   \
                        else *q = MINF(*q, val);                                                       \
                    }                                                                                  \
                }                                                                                      \
        }                                                                                              \
    } while (0)

static double add_d(double a, double b) { return a + b; }
static float add_f(float a, float b) { return a + b; }

/* The reference runs the columns of one pass on threads (src/scatterstencil.jl:56-57).  Columns of a
 * pass are 2R + 1 apart, so they write disjoint target columns and every dest cell still receives its
 * contributions in (pass, row, offset) order: the threaded run equals the one-thread run bit for bit.
 * Under Wrap that holds only when the column count is a multiple of 2R + 1 (otherwise the seam columns
 * of one pass meet, a race in the reference); those grids run on one thread. */
int orc_scatter(const stc_grid* src, const stc_grid* dst, const stc_stencil* st, const stc_scatter_op* op,
                const stc_bc* bc, int nthreads) {
    if (!src || !dst || !st || !op || !bc || src->ndims != 2 || dst->ndims != 2 || st->ndims != 2)
        return STC_ERR_UNSUPPORTED;
    if (src->dtype != dst->dtype || (src->dtype != STC_F64 && src->dtype != STC_F32)) return STC_ERR_UNSUPPORTED;
    if (op->value == STC_SCATTER_WEIGHTED && !st->weights) return STC_ERR_KERNEL_LENGTH;
    if (bc->boundary == STC_USE && bc->padding == STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    int rc = orc_update_boundary(src, st->radius, bc);
    if (rc) return rc;
    view_t v;
    rc = make_view(src, st->radius, bc->padding, &v);
    if (rc) return rc;
    const int64_t ny = v.n[0], nx = v.n[1];
    if (dst->size[0] != ny || dst->size[1] != nx) return STC_ERR_SIZE_MISMATCH;
    const int64_t stride = 2 * (int64_t)st->radius + 1;
    const int nt = (nthreads > 1 && (bc->boundary != STC_WRAP || nx % stride == 0)) ? nthreads : 1;
    if (src->dtype == STC_F64) ORC_SCATTER_BODY(double, add_d, jl_max, jl_min);
    else ORC_SCATTER_BODY(float, add_f, jl_maxf, jl_minf);
    return STC_OK;
}
