/*
 * orc_guide.c — FP64 restatement of the path-guiding network (TEST
 * INFRASTRUCTURE ONLY): the checker for the device's FP16 tensor-core
 * forward, backward and Adam kernels.  The reference has no guiding; this
 * file *is* the specification the device follows.
 *
 * Network (all layers row-major [out][in], parameters one flat float array):
 *   x (9)  = scene-normalised position (3), normal (3), outgoing direction (3)
 *   e (256)= for input i, frequency k = 0..11: sin(2^k pi x_i), cos(2^k pi x_i)
 *            at e[24 i + 2 k], e[24 i + 2 k + 1]; e[216 + i] = x_i; rest 0
 *   h1 = relu(W1 e + b1)   W1 64x256
 *   h2 = relu(W2 h1 + b2)  W2 64x64   (and W3, W4 alike)
 *   o  = W5 h4 + b5        W5 48x64 (outputs 40..47 unused)
 * Output o -> mixture of 8 von Mises-Fisher lobes; lobe l uses o[5l..5l+4]:
 *   mu_l = m / (|m| + 1e-6), m = o[5l..5l+2]
 *   kappa_l = softplus(o[5l+3]) + 0.05
 *   pi = softmax(o[5l+4] over l)
 *   v_l(w) = kappa / (2 pi (1 - exp(-2 kappa))) exp(kappa (mu.w - 1))
 *   q(w) = sum_l pi_l v_l(w)
 * Training sample: (x, w, weight); loss = -(1/n) sum_i (weight_i / mean weight) log q(w_i | x_i),
 * the one-sample estimate of the KL divergence from the weight's target
 * density (Mueller et al., "Neural Importance Sampling", 2019).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"

#define GN_IN 9
#define GN_ENC 256
#define GN_H 64
#define GN_OUT 48
#define GN_LOBES 8

/* flat parameter offsets */
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + GN_H * GN_ENC)
#define OFF_W2 (OFF_B1 + GN_H)
#define OFF_B2 (OFF_W2 + GN_H * GN_H)
#define OFF_W3 (OFF_B2 + GN_H)
#define OFF_B3 (OFF_W3 + GN_H * GN_H)
#define OFF_W4 (OFF_B3 + GN_H)
#define OFF_B4 (OFF_W4 + GN_H * GN_H)
#define OFF_W5 (OFF_B4 + GN_H)
#define OFF_B5 (OFF_W5 + GN_OUT * GN_H)
#define N_PARAMS (OFF_B5 + GN_OUT)

int32_t orc_guide_num_params(void) {
	return N_PARAMS;
}

void orc_guide_encode(const double *x, double *e) {
	memset(e, 0, sizeof(double) * GN_ENC);
	for (int i = 0; i < GN_IN; ++i) {
		for (int k = 0; k < 12; ++k) {
			double a = ldexp(x[i], k) * 3.14159265358979323846;
			e[24 * i + 2 * k] = sin(a);
			e[24 * i + 2 * k + 1] = cos(a);
		}
		e[216 + i] = x[i];
	}
}

static void dense(const float *W, const float *b, int nout, int nin, const double *in, double *out, int relu) {
	for (int o = 0; o < nout; ++o) {
		double s = b[o];
		for (int i = 0; i < nin; ++i) s += (double)W[o * nin + i] * in[i];
		out[o] = relu && s < 0 ? 0 : s;
	}
}

typedef struct {
	double e[GN_ENC], h[4][GN_H], o[GN_OUT];
} acts;

static void forward(const float *P, const float *x9, acts *a) {
	double x[GN_IN];
	for (int i = 0; i < GN_IN; ++i) x[i] = x9[i];
	orc_guide_encode(x, a->e);
	dense(P + OFF_W1, P + OFF_B1, GN_H, GN_ENC, a->e, a->h[0], 1);
	dense(P + OFF_W2, P + OFF_B2, GN_H, GN_H, a->h[0], a->h[1], 1);
	dense(P + OFF_W3, P + OFF_B3, GN_H, GN_H, a->h[1], a->h[2], 1);
	dense(P + OFF_W4, P + OFF_B4, GN_H, GN_H, a->h[2], a->h[3], 1);
	dense(P + OFF_W5, P + OFF_B5, GN_OUT, GN_H, a->h[3], a->o, 0);
}

static double softplus(double x) {
	return x > 20 ? x : log1p(exp(x));
}

typedef struct {
	double mu[GN_LOBES][3], kappa[GN_LOBES], pi[GN_LOBES], len[GN_LOBES], m[GN_LOBES][3];
} mixture;

static void to_mixture(const double *o, mixture *mx) {
	double mxw = -1e300;
	for (int l = 0; l < GN_LOBES; ++l) mxw = fmax(mxw, o[5 * l + 4]);
	double z = 0;
	for (int l = 0; l < GN_LOBES; ++l) {
		const double *m = o + 5 * l;
		double len = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) + 1e-6;
		mx->len[l] = len;
		for (int k = 0; k < 3; ++k) mx->m[l][k] = m[k], mx->mu[l][k] = m[k] / len;
		mx->kappa[l] = softplus(m[3]) + 0.05;
		mx->pi[l] = exp(m[4] - mxw);
		z += mx->pi[l];
	}
	for (int l = 0; l < GN_LOBES; ++l) mx->pi[l] /= z;
}

static double vmf(double kappa, const double *mu, const double *w) {
	double c = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
	return kappa / (2 * 3.14159265358979323846 * -expm1(-2 * kappa)) * exp(kappa * (c - 1));
}

/* outputs -> mixture pdf of direction w (for tests) */
double orc_guide_pdf(const double *o48, const double *w) {
	mixture mx;
	to_mixture(o48, &mx);
	double q = 0;
	for (int l = 0; l < GN_LOBES; ++l) q += mx.pi[l] * vmf(mx.kappa[l], mx.mu[l], w);
	return q;
}

/* raw outputs (n x 48) of the network for features (n x 9) */
void orc_guide_forward(const float *params, const float *feat, int64_t n, double *out) {
	acts *a = (acts *)malloc(sizeof(acts));
	for (int64_t i = 0; i < n; ++i) {
		forward(params, feat + GN_IN * i, a);
		memcpy(out + GN_OUT * i, a->o, sizeof(double) * GN_OUT);
	}
	free(a);
}

/* d(-log q)/d(outputs) for one sample, times its weight */
static double out_grad(const double *o, const double *w, double wt, double *g) {
	mixture mx;
	to_mixture(o, &mx);
	double v[GN_LOBES], q = 0;
	for (int l = 0; l < GN_LOBES; ++l) {
		v[l] = vmf(mx.kappa[l], mx.mu[l], w);
		q += mx.pi[l] * v[l];
	}
	memset(g, 0, sizeof(double) * GN_OUT);
	for (int l = 0; l < GN_LOBES; ++l) {
		double r = mx.pi[l] * v[l] / q; /* responsibility */
		double k = mx.kappa[l];
		double c = mx.mu[l][0] * w[0] + mx.mu[l][1] * w[1] + mx.mu[l][2] * w[2];
		/* d(-log q)/d kappa, chained through softplus */
		double dlogv = 1 / k - 2 / expm1(2 * k) + (c - 1);
		double sig = 1 / (1 + exp(-o[5 * l + 3]));
		g[5 * l + 3] = -r * dlogv * sig;
		/* d(-log q)/d mu = -r kappa w, chained through mu = m / (|m| + eps) */
		double dmu[3] = { -r * k * w[0], -r * k * w[1], -r * k * w[2] };
		double len = mx.len[l], nm = len - 1e-6;
		double mdot = dmu[0] * mx.m[l][0] + dmu[1] * mx.m[l][1] + dmu[2] * mx.m[l][2];
		for (int j = 0; j < 3; ++j) g[5 * l + j] = dmu[j] / len - (nm > 0 ? mx.m[l][j] * mdot / (nm * len * len) : 0);
		/* softmax */
		g[5 * l + 4] = mx.pi[l] - r;
	}
	for (int j = 0; j < GN_OUT; ++j) g[j] *= wt;
	return -wt * log(q);
}

static void dense_back(const float *W, int nout, int nin, const double *dz, const double *in, double *dW, double *db,
	double *din) {
	for (int o = 0; o < nout; ++o) {
		db[o] += dz[o];
		for (int i = 0; i < nin; ++i) dW[o * nin + i] += dz[o] * in[i];
	}
	if (din)
		for (int i = 0; i < nin; ++i) {
			double s = 0;
			for (int o = 0; o < nout; ++o) s += (double)W[o * nin + i] * dz[o];
			din[i] = s;
		}
}

/* samples: n x 13 (features 9, direction 3, weight 1).  Returns the mean
 * loss and the gradient of it (N_PARAMS doubles). */
double orc_guide_loss_grad(const float *params, const float *samples, int64_t n, double *grad) {
	memset(grad, 0, sizeof(double) * N_PARAMS);
	double wsum = 0;
	for (int64_t i = 0; i < n; ++i) wsum += samples[13 * i + 12];
	double wmean = wsum / (double)n;
	if (!(wmean > 0)) return 0;
	acts *a = (acts *)malloc(sizeof(acts));
	double loss = 0;
	for (int64_t i = 0; i < n; ++i) {
		const float *s = samples + 13 * i;
		forward(params, s, a);
		double w[3] = { s[9], s[10], s[11] };
		double g5[GN_OUT], d4[GN_H], d3[GN_H], d2[GN_H], d1[GN_H];
		loss += out_grad(a->o, w, s[12] / wmean / (double)n, g5);
		dense_back(params + OFF_W5, GN_OUT, GN_H, g5, a->h[3], grad + OFF_W5, grad + OFF_B5, d4);
		for (int j = 0; j < GN_H; ++j) d4[j] = a->h[3][j] > 0 ? d4[j] : 0;
		dense_back(params + OFF_W4, GN_H, GN_H, d4, a->h[2], grad + OFF_W4, grad + OFF_B4, d3);
		for (int j = 0; j < GN_H; ++j) d3[j] = a->h[2][j] > 0 ? d3[j] : 0;
		dense_back(params + OFF_W3, GN_H, GN_H, d3, a->h[1], grad + OFF_W3, grad + OFF_B3, d2);
		for (int j = 0; j < GN_H; ++j) d2[j] = a->h[1][j] > 0 ? d2[j] : 0;
		dense_back(params + OFF_W2, GN_H, GN_H, d2, a->h[0], grad + OFF_W2, grad + OFF_B2, d1);
		for (int j = 0; j < GN_H; ++j) d1[j] = a->h[0][j] > 0 ? d1[j] : 0;
		dense_back(params + OFF_W1, GN_H, GN_ENC, d1, a->e, grad + OFF_W1, grad + OFF_B1, NULL);
	}
	free(a);
	/* unused outputs 40..47 carry no gradient */
	for (int o = 40; o < GN_OUT; ++o) {
		grad[OFF_B5 + o] = 0;
		for (int i = 0; i < GN_H; ++i) grad[OFF_W5 + o * GN_H + i] = 0;
	}
	return loss;
}

/* Adam (Kingma & Ba 2015), bias-corrected, on float parameters in place. */
void orc_guide_adam(float *params, float *m, float *v, const double *grad, int64_t step, double lr, double b1, double b2,
	double eps) {
	double c1 = 1 - pow(b1, (double)step), c2 = 1 - pow(b2, (double)step);
	for (int i = 0; i < N_PARAMS; ++i) {
		double g = grad[i];
		m[i] = (float)(b1 * m[i] + (1 - b1) * g);
		v[i] = (float)(b2 * v[i] + (1 - b2) * g * g);
		params[i] = (float)(params[i] - lr * (m[i] / c1) / (sqrt(v[i] / c2) + eps));
	}
}
