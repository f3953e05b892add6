// Function-graph evaluation at integration points in one kernel.
//
// The reference evaluates its function graph point by point through C++
// virtual calls (SwarmVariableFn maps an integration point to its material
// particle, L/Underworld/Function/src/SwarmVariableFn.cpp:30-110; Map,
// Conditional, math and arithmetic nodes in L/Underworld/Function/src/*.cpp).
// Here the Python layer compiles the graph into a short register program
// (underworld2_gb300/function.py: compile_program) and every thread runs it for
// one point: inputs are read once, intermediates stay in registers, outputs are
// written once.  All threads execute the same instruction stream, so the
// interpreter's switch does not diverge.
#include <cmath>

#include "uwg_internal.cuh"

namespace {

// opcodes (function.py: _OPS)
enum : int32_t {
    OP_CONST = 0,  // r[dst] = imm
    OP_INPUT = 1,  // r[dst] = input a, component b
    OP_ADD = 2, OP_SUB = 3, OP_MUL = 4, OP_DIV = 5, OP_POW = 6, OP_MAX = 7, OP_MIN = 8,
    OP_LT = 9, OP_LE = 10, OP_GT = 11, OP_GE = 12, OP_AND = 13, OP_OR = 14, OP_XOR = 15,
    OP_NEG = 16, OP_ABS = 17, OP_EXP = 18, OP_LOG = 19, OP_LOG2 = 20, OP_LOG10 = 21, OP_SQRT = 22,
    OP_SIN = 23, OP_COS = 24, OP_TAN = 25, OP_ASIN = 26, OP_ACOS = 27, OP_ATAN = 28,
    OP_SINH = 29, OP_COSH = 30, OP_TANH = 31, OP_ASINH = 32, OP_ACOSH = 33, OP_ATANH = 34,
    OP_ERF = 35, OP_ERFC = 36,
    OP_EQK = 37,     // r[dst] = round(r[a]) == (int64)imm
    OP_SELECT = 38,  // r[dst] = r[(int)imm] != 0 ? r[a] : r[b]
    OP_CHECK = 39,   // if r[a] == 0: flag error code b
    OP_OUT = 40,     // out[i * nout + dst] = r[a]
    OP_COPY = 41,    // r[dst] = r[a]
    OP_FINITE = 42,  // if r[a] is not finite: flag error code b
};

constexpr int MAX_REG = 128;

__device__ __forceinline__ double load_input(const uwg_fn_input& in, int64_t row, int comp) {
    const int64_t k = row * in.count + comp;
    switch (in.dtype) {
        case 0: return ((const double*)in.ptr)[k];
        case 1: return (double)((const float*)in.ptr)[k];
        case 2: return (double)((const int32_t*)in.ptr)[k];
        case 3: return (double)((const int8_t*)in.ptr)[k];
        case 4: return (double)((const int16_t*)in.ptr)[k];
        default: return (double)((const int64_t*)in.ptr)[k];
    }
}

__global__ void k_fn_eval(int64_t n, int nops, const uwg_fn_op* __restrict__ ops, const uwg_fn_input* __restrict__ ins,
                          const int32_t* __restrict__ pid, int nout, int out_by_particle, double* __restrict__ out,
                          int32_t* flags) {
    extern __shared__ unsigned char fn_smem[];
    uwg_fn_op* sops = (uwg_fn_op*)fn_smem;
    for (int k = threadIdx.x; k < nops; k += blockDim.x) sops[k] = ops[k];
    __syncthreads();
    double r[MAX_REG];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t prow = pid ? (int64_t)pid[i] : i;
        for (int k = 0; k < nops; k++) {
            const uwg_fn_op o = sops[k];
            const double x = (o.a >= 0 && o.a < MAX_REG) ? r[o.a] : 0.0;
            const double y = (o.b >= 0 && o.b < MAX_REG) ? r[o.b] : 0.0;
            double v = 0.0;
            switch (o.op) {
                case OP_CONST: v = o.imm; break;
                case OP_INPUT: {
                    const uwg_fn_input in = ins[o.a];
                    v = load_input(in, in.by_particle ? prow : i, o.b);
                    break;
                }
                case OP_ADD: v = x + y; break;
                case OP_SUB: v = x - y; break;
                case OP_MUL: v = x * y; break;
                case OP_DIV: v = x / y; break;
                case OP_POW: v = pow(x, y); break;
                case OP_MAX: v = (x != x || y != y) ? NAN : fmax(x, y); break;
                case OP_MIN: v = (x != x || y != y) ? NAN : fmin(x, y); break;
                case OP_LT: v = x < y ? 1.0 : 0.0; break;
                case OP_LE: v = x <= y ? 1.0 : 0.0; break;
                case OP_GT: v = x > y ? 1.0 : 0.0; break;
                case OP_GE: v = x >= y ? 1.0 : 0.0; break;
                case OP_AND: v = (x != 0.0 && y != 0.0) ? 1.0 : 0.0; break;
                case OP_OR: v = (x != 0.0 || y != 0.0) ? 1.0 : 0.0; break;
                case OP_XOR: v = ((x != 0.0) != (y != 0.0)) ? 1.0 : 0.0; break;
                case OP_NEG: v = -x; break;
                case OP_ABS: v = fabs(x); break;
                case OP_EXP: v = exp(x); break;
                case OP_LOG: v = log(x); break;
                case OP_LOG2: v = log2(x); break;
                case OP_LOG10: v = log10(x); break;
                case OP_SQRT: v = sqrt(x); break;
                case OP_SIN: v = sin(x); break;
                case OP_COS: v = cos(x); break;
                case OP_TAN: v = tan(x); break;
                case OP_ASIN: v = asin(x); break;
                case OP_ACOS: v = acos(x); break;
                case OP_ATAN: v = atan(x); break;
                case OP_SINH: v = sinh(x); break;
                case OP_COSH: v = cosh(x); break;
                case OP_TANH: v = tanh(x); break;
                case OP_ASINH: v = asinh(x); break;
                case OP_ACOSH: v = acosh(x); break;
                case OP_ATANH: v = atanh(x); break;
                case OP_ERF: v = erf(x); break;
                case OP_ERFC: v = erfc(x); break;
                case OP_EQK: v = (llrint(x) == (long long)o.imm) ? 1.0 : 0.0; break;
                case OP_SELECT: {
                    const int c = (int)o.imm;
                    v = (c >= 0 && c < MAX_REG && r[c] != 0.0) ? x : y;
                    break;
                }
                case OP_CHECK:
                    if (x == 0.0) atomicOr(flags, 1 << (o.b & 15));
                    continue;
                case OP_FINITE:
                    if (!isfinite(x)) atomicOr(flags, 1 << (o.b & 15));
                    continue;
                case OP_OUT:
                    if (o.dst >= 0 && o.dst < nout) out[(out_by_particle ? prow : i) * nout + o.dst] = x;
                    continue;
                case OP_COPY: v = x; break;
                default: atomicOr(flags, 1 << 15); continue;
            }
            if (o.dst >= 0 && o.dst < MAX_REG) r[o.dst] = v;
        }
    }
}

}  // namespace

extern "C" int uwg_fn_eval(uwg_ctx* c, int nops, const uwg_fn_op* ops, int ninputs, const uwg_fn_input* inputs,
                           int64_t n, const int32_t* pid, int nout, int out_by_particle, double* out,
                           int32_t* flags_h) {
    if (!c || (out_by_particle && !pid) || nops < 0 || nops > 4096 || ninputs < 0 || ninputs > 256 || n < 0 || nout < 1 ||
        (n && (!ops || !out)) || (ninputs && !inputs))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_fn_eval: bad argument");
    for (int k = 0; k < nops; k++) {
        const uwg_fn_op& o = ops[k];
        if (o.op < 0 || o.op > 42 || o.dst >= 128 || o.a >= 128 || o.b >= 128 ||
            (o.op == 1 && (o.a < 0 || o.a >= ninputs || o.b < 0 || o.b >= inputs[o.a].count)))
            return uwg_set_error(c, UWG_ERR_ARG, "uwg_fn_eval: invalid program (op " + std::to_string(k) + ")");
    }
    for (int k = 0; k < ninputs; k++)
        if (!inputs[k].ptr || inputs[k].count < 1 || inputs[k].dtype < 0 || inputs[k].dtype > 5)
            return uwg_set_error(c, UWG_ERR_ARG, "uwg_fn_eval: invalid input " + std::to_string(k));
    if (flags_h) *flags_h = 0;
    if (n == 0) return UWG_OK;
    // program, inputs and the flag word in the context's reduction scratch
    size_t ob = sizeof(uwg_fn_op) * (size_t)nops, ib = sizeof(uwg_fn_input) * (size_t)ninputs;
    if (ob + ib + 64 > 4096 * sizeof(double))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_fn_eval: program too long");
    unsigned char* base = (unsigned char*)c->red;
    uwg_fn_op* dops = (uwg_fn_op*)base;
    uwg_fn_input* dins = (uwg_fn_input*)(base + ((ob + 15) & ~(size_t)15));
    int32_t* dflags = (int32_t*)(base + ((ob + 15) & ~(size_t)15) + ((ib + 15) & ~(size_t)15));
    UWG_CUDA(c, cudaMemcpyAsync(dops, ops, ob, cudaMemcpyHostToDevice, c->stream));
    if (ib) UWG_CUDA(c, cudaMemcpyAsync(dins, inputs, ib, cudaMemcpyHostToDevice, c->stream));
    UWG_CUDA(c, cudaMemsetAsync(dflags, 0, 4, c->stream));
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = std::min<int64_t>((n + 127) / 128, (int64_t)std::max(nsm, 1) * 16);
    k_fn_eval<<<(unsigned)blocks, 128, ob, c->stream>>>(n, nops, dops, dins, pid, nout, out_by_particle, out, dflags);
    UWG_CUDA(c, cudaGetLastError());
    int32_t f = 0;
    UWG_CUDA(c, cudaMemcpyAsync(&f, dflags, 4, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));   // the host copies of ops/inputs outlive their copies
    if (flags_h) *flags_h = f;
    if (f & (1 << 15)) return uwg_set_error(c, UWG_ERR_ARG, "uwg_fn_eval: unknown opcode");
    return UWG_OK;
}
