/*
 * C entry points over the reference's own PCG32 (tools/Rng.h) and CDF
 * (core/CDF.h + core/CDF.cpp), compiled in place from the reference sources
 * with oracle/ref_shim.h force-included.  Used only to pin the oracle's
 * restatement and to generate the golden fixtures in tests/golden/.
 * TEST INFRASTRUCTURE ONLY.
 */
#include "tools/Rng.h"
#include "core/CDF.h"

extern "C" {

void ref_pcg_stream(uint64_t initstate, uint64_t initseq, int n, uint32_t *out)
{
    Rng r(initstate, initseq);
    for (int i = 0; i < n; i++) out[i] = r.nextUInt();
}

void ref_pcg_reals(uint64_t initstate, uint64_t initseq, int n, float *out)
{
    Rng r(initstate, initseq);
    for (int i = 0; i < n; i++) out[i] = r.nextReal();
}

/* Build a CDF from `pdfs`, normalize it, then run sampleAndReuse on each u. */
void ref_cdf_sample_reuse(const float *pdfs, int n, const float *u, int m,
                          int *index, float *u_out, float *pdf_out, float *sum_out)
{
    CDF c;
    for (int i = 0; i < n; i++) c.add(pdfs[i]);
    *sum_out = c.getSum();
    c.normalize();
    for (int k = 0; k < m; k++) {
        real v = u[k], p;
        index[k] = c.sampleAndReuse(v, p);
        u_out[k] = v;
        pdf_out[k] = p;
    }
}

/* CDF::sample(samp, pdf) without reuse. */
void ref_cdf_sample(const float *pdfs, int n, const float *u, int m, int *index, float *pdf_out)
{
    CDF c;
    for (int i = 0; i < n; i++) c.add(pdfs[i]);
    c.normalize();
    for (int k = 0; k < m; k++) {
        real p;
        index[k] = c.sample(u[k], p);
        pdf_out[k] = p;
    }
}

}
