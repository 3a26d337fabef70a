/*
 * Oracle body: a plain-C restatement of the reference's sequential Hull-White
 * trinomial-tree pricer.  TEST INFRASTRUCTURE ONLY - it checks the product and is
 * timed as the CPU baseline; the product never links or calls it.
 *
 * Included twice by hwt_seq.c: once with REAL=double (the reference built with
 * -DUSE_DOUBLE) and once with REAL=float (the reference's default float build).
 *
 * Expression types mirror the reference's C++ exactly, because the FP32 goldens
 * depend on them: in the reference, exp/log/sqrt/ceil are called unqualified on
 * `real` values with only the C library's double overloads in scope, so in the
 * float build those calls (and every product they feed that is held in `auto`)
 * are evaluated in double and rounded to float only where the result is stored
 * in a `real`.  The comments give the reference line each statement follows.
 */

typedef REAL SFX(real);

/* common/Domain.hpp:11-46  getYieldAtYear */
static SFX(real) SFX(yield_at_year)(SFX(real) t, int term_unit, const SFX(real) *prices,
                                    const int32_t *days, int size)
{
    const int t_days = (int)ROUNDR(t * term_unit);
    int first = 0, second = 0;
    for (int i = 0; i < size; ++i) {
        const int32_t d = days[i];
        if (d >= t_days) {
            second = i;
            break;
        }
        first = i;
    }
    if (first == second) return prices[0];         /* t_days <= days[0] */
    if (first == size - 1) return prices[size - 1]; /* past the last node */
    const int32_t t1 = days[first], t2 = days[second];
    const SFX(real) p1 = prices[first], p2 = prices[second];
    const SFX(real) coefficient = (t_days - t1) / (SFX(real))(t2 - t1);
    return p1 + coefficient * (p2 - p1);
}

/* common/Domain.hpp:51-96  branching probabilities (Hull-White 1996, exhibit 1) */
static inline SFX(real) SFX(pu_a)(int j, SFX(real) M) { return (SFX(real))1 / (SFX(real))6 + (j * j * M * M + j * M) * (SFX(real))0.5; }
static inline SFX(real) SFX(pm_a)(int j, SFX(real) M) { return (SFX(real))2 / (SFX(real))3 - j * j * M * M; }
static inline SFX(real) SFX(pd_a)(int j, SFX(real) M) { return (SFX(real))1 / (SFX(real))6 + (j * j * M * M - j * M) * (SFX(real))0.5; }
static inline SFX(real) SFX(pu_b)(int j, SFX(real) M) { return (SFX(real))1 / (SFX(real))6 + (j * j * M * M - j * M) * (SFX(real))0.5; }
static inline SFX(real) SFX(pm_b)(int j, SFX(real) M) { return -(SFX(real))1 / (SFX(real))3 - j * j * M * M + (SFX(real))2 * j * M; }
static inline SFX(real) SFX(pd_b)(int j, SFX(real) M) { return (SFX(real))7 / (SFX(real))6 + (j * j * M * M - (SFX(real))3 * j * M) * (SFX(real))0.5; }
static inline SFX(real) SFX(pu_c)(int j, SFX(real) M) { return (SFX(real))7 / (SFX(real))6 + (j * j * M * M + (SFX(real))3 * j * M) * (SFX(real))0.5; }
static inline SFX(real) SFX(pm_c)(int j, SFX(real) M) { return -(SFX(real))1 / (SFX(real))3 - j * j * M * M - (SFX(real))2 * j * M; }
static inline SFX(real) SFX(pd_c)(int j, SFX(real) M) { return (SFX(real))1 / (SFX(real))6 + (j * j * M * M + j * M) * (SFX(real))0.5; }

/* common/OptionConstants.hpp:14-54  per-option constants */
typedef struct {
    SFX(real) t, dt, dr, X, M;
    int32_t jmax, n, width;
    uint16_t term_unit;
    int8_t type;
} SFX(consts);

static void SFX(make_consts)(SFX(consts) *c, SFX(real) strike, SFX(real) bond_maturity,
                             SFX(real) option_maturity, uint16_t term_unit, uint16_t term_steps,
                             SFX(real) a, SFX(real) sigma, int8_t type)
{
    c->term_unit = term_unit;
    const SFX(real) T = bond_maturity;
    const int units_per_year = (int)ceil((double)((SFX(real))365 / term_unit)); /* :33 */
    c->n = (int32_t)(term_steps * units_per_year * T);                          /* :35 */
    c->t = option_maturity;                                                     /* :36 */
    c->dt = units_per_year / (SFX(real))term_steps;                             /* :37 */
    c->type = type;
    c->X = strike;
    /* :43-45  V and the exp() results are double in both builds */
    const double V = sigma * sigma * ((SFX(real))1 - exp((double)(-(SFX(real))2 * a * c->dt))) / ((SFX(real))2 * a);
    c->dr = (SFX(real))sqrt((SFX(real))3 * V);
    c->M = (SFX(real))(exp((double)(-a * c->dt)) - (SFX(real))1);
    c->jmax = (int)(-(SFX(real))0.184 / c->M) + 1;                              /* :51 */
    c->width = 2 * c->jmax + 1;                                                 /* :52 */
}

/* common/Domain.hpp:147-169  computeCallValue */
static inline SFX(real) SFX(call_value)(int is_maturity, SFX(real) X, int8_t type, SFX(real) res)
{
    SFX(real) ret = res;
    if (is_maturity) {
        /* std::max(a, 0) is (a < 0) ? 0 : a, which keeps a NaN */
        if (type == 1) ret = (X - res) < 0 ? (SFX(real))0 : (X - res);      /* PUT  */
        else if (type == 0) ret = (res - X) < 0 ? (SFX(real))0 : (res - X); /* CALL */
    }
    if (ret == (SFX(real))INFINITY) return REALMAX;
    if (ret == -(SFX(real))INFINITY) return REALMIN;
    return ret;
}

/* seq/Seq.hpp:24-179  computeSingleOption; scratch rows are caller-provided */
static SFX(real) SFX(price_one)(const SFX(consts) *c, const SFX(real) *yp, const int32_t *yd,
                                int ysize, SFX(real) *scratch)
{
    const int W = c->width, jmax = c->jmax, jmin = -jmax;
    SFX(real) *rate = scratch, *pu = rate + W, *pm = pu + W, *pd = pm + W;
    SFX(real) *Qs = pd + W, *QsCopy = Qs + W, *alphas = QsCopy + W;

    /* :26-50 precomputed probabilities and rates */
    rate[0] = jmin * c->dr;
    pu[0] = SFX(pu_b)(jmin, c->M); pm[0] = SFX(pm_b)(jmin, c->M); pd[0] = SFX(pd_b)(jmin, c->M);
    rate[W - 1] = jmax * c->dr;
    pu[W - 1] = SFX(pu_c)(jmax, c->M); pm[W - 1] = SFX(pm_c)(jmax, c->M); pd[W - 1] = SFX(pd_c)(jmax, c->M);
    for (int i = 1; i < W - 1; ++i) {
        const int j = i + jmin;
        rate[i] = j * c->dr;
        pu[i] = SFX(pu_a)(j, c->M); pm[i] = SFX(pm_a)(j, c->M); pd[i] = SFX(pd_a)(j, c->M);
    }

    /* :53-58 */
    for (int i = 0; i < W; ++i) Qs[i] = QsCopy[i] = 0;
    Qs[jmax] = 1;
    for (int i = 0; i <= c->n; ++i) alphas[i] = 0;
    alphas[0] = SFX(yield_at_year)(c->dt, c->term_unit, yp, yd, ysize);

    /* :60-113 forward induction */
    for (int i = 0; i < c->n; ++i) {
        const int jhigh = i < jmax ? i : jmax;
        const SFX(real) alpha = alphas[i];
        for (int j = -jhigh; j <= jhigh; ++j) {
            const int k = j - jmin;
            const double qexp = Qs[k] * exp((double)(-(alpha + rate[k]) * c->dt)); /* :70 */
            if (j == jmin) {
                QsCopy[k + 2] += pu[k] * qexp;
                QsCopy[k + 1] += pm[k] * qexp;
                QsCopy[k] += pd[k] * qexp;
            } else if (j == jmax) {
                QsCopy[k] += pu[k] * qexp;
                QsCopy[k - 1] += pm[k] * qexp;
                QsCopy[k - 2] += pd[k] * qexp;
            } else {
                QsCopy[k + 1] += pu[k] * qexp;
                QsCopy[k] += pm[k] * qexp;
                QsCopy[k - 1] += pd[k] * qexp;
            }
        }
        /* :97-106 alpha fit against the curve's discount factor */
        const int jhigh1 = (i + 1) < jmax ? (i + 1) : jmax;
        SFX(real) alpha_val = 0;
        for (int j = -jhigh1; j <= jhigh1; ++j) {
            const int k = j - jmin;
            alpha_val += QsCopy[k] * exp((double)(-rate[k] * c->dt));
        }
        {   /* common/Domain.hpp:98-104 computeAlpha */
            const SFX(real) ti = (i + 2) * c->dt;
            const SFX(real) R = SFX(yield_at_year)(ti, c->term_unit, yp, yd, ysize);
            const double P = exp((double)(-R * ti));
            alphas[i + 1] = (SFX(real))(log(alpha_val / P) / c->dt);
        }
        SFX(real) *tmp = Qs; Qs = QsCopy; QsCopy = tmp;
        for (int k = 0; k < W; ++k) QsCopy[k] = 0;
    }

    /* :115-169 backward induction */
    SFX(real) *call = Qs, *callCopy = QsCopy;
    for (int k = 0; k < W; ++k) call[k] = 100;
    const int maturity_step = (int)(c->t / c->dt); /* :125 */
    for (int i = c->n - 1; i >= 0; --i) {
        const int jhigh = i < jmax ? i : jmax;
        const SFX(real) alpha = alphas[i];
        const int is_maturity = (i == maturity_step);
        for (int j = -jhigh; j <= jhigh; ++j) {
            const int k = j - jmin;
            const double call_exp = exp((double)(-(alpha + rate[k]) * c->dt));
            SFX(real) res;
            if (j == jmax)
                res = (SFX(real))((pu[k] * call[k] + pm[k] * call[k - 1] + pd[k] * call[k - 2]) * call_exp);
            else if (j == jmin)
                res = (SFX(real))((pu[k] * call[k + 2] + pm[k] * call[k + 1] + pd[k] * call[k]) * call_exp);
            else
                res = (SFX(real))((pu[k] * call[k + 1] + pm[k] * call[k] + pd[k] * call[k - 1]) * call_exp);
            callCopy[k] = SFX(call_value)(is_maturity, c->X, c->type, res);
        }
        SFX(real) *tmp = call; call = callCopy; callCopy = tmp;
        for (int k = 0; k < W; ++k) callCopy[k] = 0;
    }
    return call[jmax];
}

/* seq/Seq.hpp:181-190  computeOptions: OpenMP over options (static schedule, as
 * the reference's `#pragma omp parallel for`).  threads <= 0 keeps the OpenMP
 * default.  Returns 0, or -1 if scratch memory could not be allocated. */
int SFX(oracle_price)(int n_options, const SFX(real) *strike, const SFX(real) *bond_maturity,
                      const SFX(real) *option_maturity, const uint16_t *term_unit,
                      const uint16_t *term_steps, const SFX(real) *a, const SFX(real) *sigma,
                      const int8_t *type, int yield_n, const SFX(real) *yield_rate,
                      const int32_t *yield_day, SFX(real) *out, int threads)
{
    int failed = 0;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for reduction(| : failed)
    for (int i = 0; i < n_options; ++i) {
        SFX(consts) c;
        SFX(make_consts)(&c, strike[i], bond_maturity[i], option_maturity[i], term_unit[i],
                         term_steps[i], a[i], sigma[i], type[i]);
        SFX(real) *scratch = (SFX(real) *)malloc(sizeof(SFX(real)) * ((size_t)6 * c.width + c.n + 1 + 8));
        if (!scratch) {
            failed |= 1;
            continue;
        }
        out[i] = SFX(price_one)(&c, yield_rate, yield_day, yield_n, scratch);
        free(scratch);
    }
    return failed ? -1 : 0;
}

/* Per-option tree shape as the reference computes it (OptionConstants.hpp:29-53,
 * Seq.hpp:125): jmax, n (height), width and the maturity step (int)(t/dt). */
void SFX(oracle_shape)(int n_options, const SFX(real) *bond_maturity, const SFX(real) *option_maturity,
                       const uint16_t *term_unit, const uint16_t *term_steps, const SFX(real) *a,
                       const SFX(real) *sigma, int32_t *jmax, int32_t *n, int32_t *width,
                       int32_t *maturity_step)
{
    for (int i = 0; i < n_options; ++i) {
        SFX(consts) c;
        SFX(make_consts)(&c, 0, bond_maturity[i], option_maturity[i], term_unit[i], term_steps[i],
                         a[i], sigma[i], 0);
        jmax[i] = c.jmax;
        n[i] = c.n;
        width[i] = c.width;
        maturity_step[i] = (int)(c.t / c.dt);
    }
}
