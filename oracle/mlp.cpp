/* oracle/mlp.cpp — CPU restatement of the radiance-cache MLP (forward pass and
 * gradients of one training step).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the tensor-core kernels in mlp.cu.
 *
 * The network and its encoding are the library's own (no reference
 * counterpart): 96 encoded inputs, 5 hidden layers of 64 ReLU units, 3 linear
 * outputs (stored 16 wide).  Values are rounded to bf16 at the points where the
 * kernels hand them to the tensor cores — the encoded inputs, every hidden
 * activation, every backward gradient tile and the weights — and products are
 * summed in double precision (the tensor cores sum in fp32, so results agree
 * to rounding). */
#include "oracle.h"
#include "fmath.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int IN = 96, HID = 64, OUTP = 16, OUT = 3, LAYERS = 6, BANDS = 12;
inline int in_of(int l) { return l == 0 ? IN : HID; }
inline int out_of(int l) { return l == LAYERS - 1 ? OUTP : HID; }
inline int w_off(int l) { int o = 0; for (int k = 0; k < l; ++k) o += out_of(k) * in_of(k) + out_of(k); return o; }
inline int b_off(int l) { return w_off(l) + out_of(l) * in_of(l); }
constexpr int PARAMS = 23888;

inline float bf16(float x) {                         /* round to nearest even */
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
inline float relu(float x) { return x > 0.0f ? x : 0.0f; }

void encode(const float *q, const float *lo, const float *inv, float *f) {
    float u[3];
    for (int a = 0; a < 3; ++a) {
        float v = (q[a] - lo[a]) * inv[a];
        u[a] = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
        float s, c;                                  /* band k = sin / cos of pi 2^k u, by doubling */
        of_sincos(u[a] * 3.141592653589793f, &s, &c);
        for (int k = 0; k < BANDS; ++k) {
            f[24 * a + 2 * k] = s;
            f[24 * a + 2 * k + 1] = c;
            const float s2 = (2.0f * s) * c, c2 = c * c - s * s;
            s = s2;
            c = c2;
        }
    }
    for (int k = 0; k < 9; ++k) f[72 + k] = q[3 + k];
    for (int a = 0; a < 3; ++a) f[81 + a] = u[a];
    for (int k = 84; k < IN; ++k) f[k] = 0.0f;
}

struct Net {
    std::vector<float> w[LAYERS];    /* bf16-rounded weights [out][in] */
    std::vector<float> b[LAYERS];
    explicit Net(const float *p) {
        for (int l = 0; l < LAYERS; ++l) {
            w[l].resize((size_t)out_of(l) * in_of(l));
            b[l].resize(out_of(l));
            for (size_t k = 0; k < w[l].size(); ++k) w[l][k] = bf16(p[w_off(l) + k]);
            for (int o = 0; o < out_of(l); ++o) b[l][o] = p[b_off(l) + o];
        }
    }
};

/* acts[0] = bf16 inputs, acts[l] = bf16 outputs of layer l-1 (l = 1..5); y = outputs */
void forward(const Net &net, const float *x0, std::vector<float> *acts, float *y) {
    acts[0].assign(x0, x0 + IN);
    for (int l = 0; l < LAYERS; ++l) {
        const int nin = in_of(l), nout = out_of(l);
        std::vector<float> out(nout);
        for (int o = 0; o < nout; ++o) {
            double s = 0.0;
            for (int i = 0; i < nin; ++i) s += (double)net.w[l][(size_t)o * nin + i] * (double)acts[l][i];
            out[o] = (float)s + net.b[l][o];
        }
        if (l < LAYERS - 1) {
            acts[l + 1].resize(nout);
            for (int o = 0; o < nout; ++o) acts[l + 1][o] = bf16(relu(out[o]));
        } else {
            for (int c = 0; c < OUT; ++c) y[c] = out[c];
        }
    }
}

}  // namespace

extern "C" {

void orc_mlp_encode(const float *q12, const float *lo3, const float *inv3, float *out96) { encode(q12, lo3, inv3, out96); }

void orc_mlp_forward(const float *params, const float *lo3, const float *inv3, const float *q12, uint32_t n,
                     float *out3) {
    Net net(params);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        float f[IN];
        encode(q12 + 12 * i, lo3, inv3, f);
        for (int k = 0; k < IN; ++k) f[k] = bf16(f[k]);
        std::vector<float> acts[LAYERS];
        forward(net, f, acts, out3 + 3 * i);
    }
}

/* Gradient of the mean relative L2 loss over n samples (16 floats each: query,
 * target, weight) and the loss sum, as one training step computes them. */
void orc_mlp_grad(const float *params, const float *lo3, const float *inv3, const float *samples, uint32_t n,
                  double *grad, double *loss_out) {
    Net net(params);
    uint32_t valid = 0;
    for (uint32_t i = 0; i < n; ++i) valid += samples[16 * (size_t)i + 15] > 0.0f ? 1u : 0u;
    const float scale = 1.0f / (3.0f * (float)(valid ? valid : 1u));
    std::vector<double> g(PARAMS, 0.0);
    double loss = 0.0;
    for (uint32_t s = 0; s < n; ++s) {
        const float *sm = samples + 16 * (size_t)s;
        const float wgt = sm[15];
        float f[IN];
        if (wgt > 0.0f) encode(sm, lo3, inv3, f);
        else for (int k = 0; k < IN; ++k) f[k] = 0.0f;
        for (int k = 0; k < IN; ++k) f[k] = bf16(f[k]);
        std::vector<float> acts[LAYERS];
        float y[OUT];
        forward(net, f, acts, y);
        /* output gradient, rounded as the kernel hands it to the tensor cores */
        std::vector<float> gl(OUTP, 0.0f);
        for (int c = 0; c < OUT; ++c) {
            const float e = y[c] - sm[12 + c], den = y[c] * y[c] + 0.01f;
            loss += (double)(wgt * ((e * e) / den));
            gl[c] = bf16(wgt * (2.0f * e / den) * scale);
        }
        for (int l = LAYERS - 1; l >= 0; --l) {
            const int nin = in_of(l), nout = out_of(l);
            for (int o = 0; o < nout; ++o) {
                if (gl[o] == 0.0f) continue;
                for (int i = 0; i < nin; ++i) g[w_off(l) + o * nin + i] += (double)gl[o] * (double)acts[l][i];
                g[b_off(l) + o] += (double)gl[o];
            }
            if (l == 0) break;
            std::vector<float> gp(nin);
            for (int i = 0; i < nin; ++i) {
                double sum = 0.0;
                for (int o = 0; o < nout; ++o) sum += (double)gl[o] * (double)net.w[l][(size_t)o * nin + i];
                gp[i] = bf16(acts[l][i] != 0.0f ? (float)sum : 0.0f);
            }
            gl.swap(gp);
        }
    }
    for (int p = 0; p < PARAMS; ++p) grad[p] = g[p];
    *loss_out = loss;
}

}  /* extern "C" */
