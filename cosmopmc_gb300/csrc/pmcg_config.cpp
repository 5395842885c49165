// pmcg_config.cpp — the device posterior of a CosmoPMC configuration.
//
// The reference's driver evaluates posterior_log_pdf_common
// (wrappers/src/param.c:958-1041) on its parsed configuration (config_base):
// the flat box prior, one likelihood per data set, the special prior of the
// first data set and an optional prior over a parameter subset. This file
// builds the same composition from the configuration's plain values (par_t
// codes, box, data types and their states) as a pmcg_posterior whose terms
// run on the GPU. Host code only: no per-sample computation here.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pmcg.h"
#include "pmcg_internal.h"

using pmcg::set_error;

namespace {

// par_t codes (tools/include/par.h:11-33) that change the SN Ia model but have
// no counterpart in the device plugin (likeli_SNIa, wrappers/src/sn.c:167-224).
bool sn_unsupported(int code) {
  switch (code) {
    case 4: case 5: case 6:                                   // Omega_nu_mass, Omega_c, Omega_K
    case 7: case 8: case 9: case 10: case 11: case 12: case 13:  // physical densities omega_X
    case 15: case 16:                                         // w1_de, polynomial dark energy
    case 40: case 41: case 42: case 43:                       // beta_z, log beta, stretch, colour offsets
    case 44: case 45: case 46: case 47: case 48: case 49: case 50: case 51:  // Theta1
    case 52:                                                  // beta_d (dust)
      return true;
    default:
      return false;
  }
}

// One SN Ia data set: the parameter mapping of likeli_SNIa (sn.c:167-224), the
// -M and -beta storage of the SN parameter file (par_files/cosmo_SN.par:9),
// the flatness rule of set_base_parameters (param.c:1544-1656: Omega_de given
// -> Omega_K = 1 - Omega_m - Omega_de, absent -> flat) and the SALT stretch
// form mu = m - M + alpha (s - 1) - beta c (Manual/manual.tex:1290-1295).
bool add_snia(pmcg_posterior *p, int npar, const int *par, const pmcg_snia_config *cfg, error **err) {
  if (!cfg || cfg->nsn < 1 || !cfg->z || !cfg->m || !cfg->s || !cfg->c || !cfg->cov6) {
    set_error(err, PMCG_EARG, __LINE__, "SN Ia data set: sample missing");
    return false;
  }
  pmcg_sn_data sd;
  std::memset(&sd, 0, sizeof(sd));
  sd.ip_Omegam = sd.ip_Omegade = sd.ip_w0 = sd.ip_M = sd.ip_alpha = sd.ip_beta = -1;
  bool has_om = false, has_ob = false;
  for (int i = 0; i < npar; i++) {
    const int code = par[i];
    if (sn_unsupported(code)) {
      set_error(err, PMCG_EUNSUPPORTED, __LINE__,
                "SN Ia: parameter #%d (par_t code %d) is not modelled by the device SN plugin", i, code);
      return false;
    }
    switch (code) {
      case PMCG_P_OMEGAM: sd.ip_Omegam = i; has_om = true; break;
      case 1: has_ob = true; break;              // Omega_b: no effect on distances with Omega_m given
      case PMCG_P_OMEGADE: sd.ip_Omegade = i; break;
      case PMCG_P_H100: break;                   // absorbed in M (Manual/manual.tex:1321-1322)
      case PMCG_P_W0DE: sd.ip_w0 = i; break;
      case PMCG_P_M: sd.ip_M = i; sd.neg_M = 1; break;
      case PMCG_P_ALPHA: sd.ip_alpha = i; break;
      case PMCG_P_BETA: sd.ip_beta = i; sd.neg_beta = 1; break;
      default: break;                            // parameters of other data sets
    }
  }
  if (has_ob && !has_om) {
    set_error(err, PMCG_EUNSUPPORTED, __LINE__, "SN Ia: Omega_b without Omega_m is not modelled");
    return false;
  }
  // the sample: x1 = s - 1 (the stretch form); the covariance of (m, s, c)
  // is that of (m, x1, c)
  const int n = cfg->nsn;
  std::vector<double> x1(n);
  for (int i = 0; i < n; i++) x1[i] = cfg->s[i] - 1.0;
  sd.nsn = n;
  sd.z = cfg->z;
  sd.mB = cfg->m;
  sd.x1 = x1.data();
  sd.c = cfg->c;
  sd.cov6 = cfg->cov6;
  sd.sig_int = cfg->sig_int;
  sd.v_pec = cfg->v_pec;
  sd.h = cfg->h > 0.0 ? cfg->h : 0.7;
  sd.chi2mode = cfg->chi2mode;
  sd.add_logdet = cfg->add_logdetCov;
  sd.quad_nodes = cfg->quad_nodes > 0 ? cfg->quad_nodes : 4;
  sd.def_Omegam = cfg->Omega_m;
  sd.def_w0 = cfg->w0_de;
  sd.def_M = -cfg->Theta2[0];
  sd.def_alpha = cfg->Theta2[1];
  sd.def_beta = -cfg->Theta2[2];
  pmcg_posterior_add_snia(p, &sd, err);
  return !isError(*err);
}

// An Mvdens data set (likeli_Mvdens, param.c:1485-1493): one component of weight 1.
bool add_mvdens(pmcg_posterior *p, const mvdens *g, error **err) {
  if (!g || g->ndim < 1) {
    set_error(err, PMCG_EARG, __LINE__, "Mvdens data set: density missing");
    return false;
  }
  mix_mvdens *m = mix_mvdens_alloc(1, g->ndim, err);
  if (!m) return false;
  const int d = g->ndim;
  m->wght[0] = 1.0;
  mvdens *c = m->comp[0];
  c->df = g->df;
  c->chol = g->chol;
  c->det = g->det;
  c->band_limit = g->band_limit;
  std::memcpy(c->mean, g->mean, sizeof(double) * d);
  std::memcpy(c->std, g->std, sizeof(double) * d * d);
  pmcg_posterior_add_mixmvdens(p, m, err);
  mix_mvdens_free(&m);
  return !isError(*err);
}

}  // namespace

// Moves a local error chain to the front of the caller's (or drops it).
static void forward_chain(error *le, error **err) {
  if (!le) return;
  if (!err) {
    purgeError(&le);
    return;
  }
  error *tail = le;
  while (tail->next) tail = tail->next;
  tail->next = *err;
  *err = le;
}

extern "C" pmcg_posterior *pmcg_posterior_from_config(int npar, const int *par, const double *min, const double *max,
                                                      int ndata, const int *data, const void *const *data_state,
                                                      const mvdens *prior, const int *indprior, double a_acc,
                                                      error **err) {
  if (npar < 1 || !par || !min || !max || ndata < 1 || !data || !data_state) {
    set_error(err, PMCG_EARG, __LINE__, "pmcg_posterior_from_config: missing argument");
    return nullptr;
  }
  // every step reports into a local chain, so a failure is seen whether or not
  // the caller passed an error pointer
  error *le = nullptr;
  pmcg_posterior *p = pmcg_posterior_alloc(npar, min, max, &le);
  int special = PMCG_SPECIAL_NONE, n_sn = 0;
  for (int d = 0; p && d < ndata && !isError(le); d++) {
    switch (data[d]) {
      case PMCG_DATA_MIXMVDENS:
        if (!data_state[d]) set_error(&le, PMCG_EARG, __LINE__, "MixMvdens data set: mixture missing");
        else pmcg_posterior_add_mixmvdens(p, (const mix_mvdens *)data_state[d], &le);
        break;
      case PMCG_DATA_MVDENS:
        add_mvdens(p, (const mvdens *)data_state[d], &le);
        break;
      case PMCG_DATA_SNIA:
        if (n_sn++ > 0) {
          set_error(&le, PMCG_EUNSUPPORTED, __LINE__, "more than one SN Ia data set");
          break;
        }
        // the special prior is the first data set's (get_special(config->data[0], ...), param.c:998)
        if (add_snia(p, npar, par, (const pmcg_snia_config *)data_state[d], &le) && d == 0)
          special = ((const pmcg_snia_config *)data_state[d])->special;
        break;
      default:
        set_error(&le, PMCG_EUNSUPPORTED, __LINE__, "data set #%d: type %d has no device plugin", d, data[d]);
        break;
    }
  }
  if (p && !isError(le) && special != PMCG_SPECIAL_NONE) {
    int i0 = -1, i1 = -1;
    for (int i = 0; i < npar; i++) {
      if (par[i] == PMCG_P_W0DE) i0 = i;
      if (par[i] == 15) i1 = i;   // p_w1de
    }
    pmcg_posterior_set_special(p, special, i0, i1, a_acc, &le);
  }
  if (p && !isError(le) && prior) pmcg_posterior_add_mvdens_prior(p, prior, indprior, &le);
  if (isError(le) || !p) {
    if (p) pmcg_posterior_free(&p);
    forward_chain(le, err);
    return nullptr;
  }
  purgeError(&le);
  return p;
}
