/*
 * ammsb_oracle_impl.h -- precision-generic body of the oracle's hot-path
 * arithmetic.  Included twice by ammsb_oracle.c (REAL = float, double).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Every loop keeps the reference's accumulation order so that the float
 * instance reproduces the reference's rounding (modulo the neighbour
 * iteration order, which the caller supplies explicitly).
 */

/* MCMCSamplerStochastic::update_phi, mcmc_sampler_stochastic.cc:269-313 */
void SFX(oracle_update_phi)(int32_t K, const REAL *pi, REAL *phi_i, int32_t i,
                            const int32_t *nbrs, const uint8_t *y,
                            int32_t n_nbrs, const REAL *beta, REAL alpha,
                            REAL epsilon, REAL eps_t, int64_t N,
                            int64_t num_node_sample, const REAL *noise) {
  REAL phi_i_sum = R(0.0); /* np::sum: accumulate from 0 in k order */
  for (int32_t k = 0; k < K; ++k) phi_i_sum += phi_i[k];
  REAL *grads = (REAL *)calloc((size_t)K, sizeof(REAL));
  REAL *probs = (REAL *)malloc(sizeof(REAL) * (size_t)K);
  const REAL *pi_i = pi + (int64_t)i * K;
  for (int32_t n = 0; n < n_nbrs; ++n) {
    int32_t neighbor = nbrs[n];
    if (i == neighbor) continue;
    int y_ab = y[n] ? 1 : 0;
    const REAL *pi_j = pi + (int64_t)neighbor * K;
    REAL e = (y_ab == 1) ? epsilon : (R(1.0) - epsilon);
    for (int32_t k = 0; k < K; ++k) {
      REAL f = (y_ab == 1) ? (beta[k] - epsilon) : (epsilon - beta[k]);
      probs[k] = pi_i[k] * (pi_j[k] * f + e);
    }
    REAL prob_sum = R(0.0);
    for (int32_t k = 0; k < K; ++k) prob_sum += probs[k];
    for (int32_t k = 0; k < K; ++k)
      grads[k] += (probs[k] / prob_sum) / phi_i[k] - R(1.0) / phi_i_sum;
  }
  REAL Nn = (R(1.0) * (REAL)N) / (REAL)num_node_sample;
  for (int32_t k = 0; k < K; ++k) {
    REAL v = RABS((phi_i[k] + eps_t / R(2.0) * (alpha - phi_i[k] + Nn * grads[k])) +
                  RSQRT(eps_t * phi_i[k]) * noise[k]);
    if (v < GUARD) v = GUARD;
    phi_i[k] = v;
  }
  free(probs);
  free(grads);
}

/* np::normalize, np.h:39-56 */
void SFX(oracle_normalize)(int32_t K, const REAL *phi_i, REAL *pi_i) {
  REAL s = R(0.0);
  for (int32_t k = 0; k < K; ++k) s += phi_i[k];
  for (int32_t k = 0; k < K; ++k) pi_i[k] = phi_i[k] / s;
}

/* MCMCSamplerStochastic::update_beta, mcmc_sampler_stochastic.cc:200-267,
 * in its two halves: the gradient summed over the minibatch edges in their
 * order (cc:212-240; grads K x 2, zeroed first) ... */
void SFX(oracle_beta_grads)(int32_t K, const REAL *pi, const int32_t *ea,
                            const int32_t *eb, const uint8_t *ey,
                            int32_t n_edges, const REAL *theta,
                            const REAL *beta, REAL epsilon, REAL *grads) {
  REAL *probs = (REAL *)malloc(sizeof(REAL) * (size_t)K);
  REAL *theta_sum = (REAL *)malloc(sizeof(REAL) * (size_t)K);
  for (int32_t k = 0; k < 2 * K; ++k) grads[k] = R(0.0);
  for (int32_t k = 0; k < K; ++k)
    theta_sum[k] = R(0.0) + theta[2 * k] + theta[2 * k + 1];
  for (int32_t ed = 0; ed < n_edges; ++ed) {
    int y = ey[ed] ? 1 : 0;
    const REAL *pa = pi + (int64_t)ea[ed] * K;
    const REAL *pb = pi + (int64_t)eb[ed] * K;
    REAL pi_sum = R(0.0);
    for (int32_t k = 0; k < K; ++k) {
      pi_sum += pa[k] * pb[k];
      REAL f = pa[k] * pb[k];
      probs[k] = (y == 1) ? beta[k] * f : (R(1.0) - beta[k]) * f;
    }
    REAL prob_0 = ((y == 1) ? epsilon : (R(1.0) - epsilon)) * (R(1.0) - pi_sum);
    REAL prob_sum = R(0.0);
    for (int32_t k = 0; k < K; ++k) prob_sum += probs[k];
    prob_sum += prob_0;
    for (int32_t k = 0; k < K; ++k) {
      REAL f = probs[k] / prob_sum;
      REAL one_over_theta_sum = R(1.0) / theta_sum[k];
      grads[2 * k] += f * ((R(1.0) - (REAL)y) / theta[2 * k] - one_over_theta_sum);
      grads[2 * k + 1] += f * ((REAL)y / theta[2 * k + 1] - one_over_theta_sum);
    }
  }
  free(theta_sum);
  free(probs);
}

/* ... and the SGRLD step of theta with those gradients, then beta
 * (cc:244-266) */
void SFX(oracle_theta_step)(int32_t K, REAL *theta, REAL *beta, const REAL *eta,
                            REAL eps_t, REAL scale, const REAL *noise,
                            const REAL *grads) {
  for (int32_t k = 0; k < K; ++k) {
    for (int c = 0; c < 2; ++c) {
      REAL th = theta[2 * k + c];
      REAL f = RSQRT(eps_t * th);
      REAL v = RABS(th + eps_t / R(2.0) * (eta[c] - th + scale * grads[2 * k + c]) +
                    f * noise[2 * k + c]);
      if (v < GUARD) v = GUARD;
      theta[2 * k + c] = v;
    }
  }
  /* np::row_normalize then SelectColumn(1) */
  for (int32_t k = 0; k < K; ++k) {
    REAL s = R(0.0) + theta[2 * k] + theta[2 * k + 1];
    beta[k] = theta[2 * k + 1] / s;
  }
}

void SFX(oracle_update_beta)(int32_t K, const REAL *pi, const int32_t *ea,
                             const int32_t *eb, const uint8_t *ey,
                             int32_t n_edges, REAL *theta, REAL *beta,
                             const REAL *eta, REAL epsilon, REAL eps_t,
                             REAL scale, const REAL *noise, REAL *grads_out) {
  REAL *grads = (REAL *)calloc(2 * (size_t)K, sizeof(REAL));
  SFX(oracle_beta_grads)(K, pi, ea, eb, ey, n_edges, theta, beta, epsilon, grads);
  if (grads_out)
    for (int32_t k = 0; k < 2 * K; ++k) grads_out[k] = grads[k];
  SFX(oracle_theta_step)(K, theta, beta, eta, eps_t, scale, noise, grads);
  free(grads);
}

/* Learner::cal_edge_likelihood, learner.h:100-139 (DONT_FOLD_Y branch) */
REAL SFX(oracle_edge_likelihood)(int32_t K, const REAL *pa, const REAL *pb,
                                 int y, const REAL *beta, REAL epsilon) {
  REAL s = R(0.0);
  if (y) {
    for (int32_t k = 0; k < K; ++k) s += pa[k] * pb[k] * beta[k];
  } else {
    REAL sum = R(0.0);
    for (int32_t k = 0; k < K; ++k) {
      REAL f = pa[k] * pb[k];
      s += f * (R(1.0) - beta[k]);
      sum += f;
    }
    s += (R(1.0) - sum) * (R(1.0) - epsilon);
  }
  if (s < R(1.0e-30)) s = R(1.0e-30);
  return s;
}

/* Learner::cal_perplexity, learner.cc:138-183 */
REAL SFX(oracle_perplexity)(int32_t K, const REAL *pi, const int32_t *ha,
                            const int32_t *hb, const uint8_t *hy, int64_t H,
                            const REAL *beta, REAL epsilon, REAL *ppx,
                            uint64_t average_count) {
  REAL link_likelihood = R(0.0), non_link_likelihood = R(0.0);
  uint64_t link_count = 0, non_link_count = 0;
  for (int64_t e = 0; e < H; ++e) {
    REAL p = SFX(oracle_edge_likelihood)(K, pi + (int64_t)ha[e] * K,
                                         pi + (int64_t)hb[e] * K, hy[e], beta,
                                         epsilon);
    ppx[e] = (ppx[e] * (REAL)(average_count - 1) + p) / (REAL)average_count;
    if (hy[e]) {
      link_count++;
      link_likelihood += RLOG(ppx[e]);
    } else {
      non_link_count++;
      non_link_likelihood += RLOG(ppx[e]);
    }
  }
  REAL avg = R(0.0);
  if (link_count + non_link_count != 0)
    avg = (link_likelihood + non_link_likelihood) /
          (REAL)(link_count + non_link_count);
  return -avg;
}
