"""CPU oracle for the edward_gb300 hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
package: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, and only as the checker or as the timed CPU
baseline, never as the thing measured or shipped.

What it restates (reference paths are relative to the blei-lab/edward tree,
version 1.3.5):

* ``philox``     -- Philox4x32-10 counter-based RNG and the Box-Muller /
                    uniform mappings the CUDA kernels use for eps, momenta
                    and the Metropolis uniform (replaces ``tf.random_normal``
                    / ``tf.random_uniform`` at ``edward/inferences/hmc.py:91,108``
                    and the reparameterised draw ``qz_copy.value()`` at
                    ``edward/inferences/klqp.py:727-731``).
* ``densities``  -- Normal / Bernoulli(logits) / HalfNormal log densities,
                    Normal-Normal KL, softplus bijector (the TF 1.x
                    distribution math inherited through
                    ``edward/models/random_variables.py:13-28``).
* ``glm``        -- log-joint and gradient of the generalised linear model
                    family (``ed.dot`` GEMV, ``edward/util/tensorflow.py:10-47``).
* ``klqp``       -- reparameterisation (analytic-KL and Monte Carlo KL) and
                    score-function ELBO gradients plus TF's Adam and the
                    default staircase learning-rate schedule
                    (``klqp.py:642-906``, ``variational_inference.py:83-121``).
* ``hmc``        -- one leapfrog + Metropolis update per chain
                    (``hmc.py:61-130,195-210``).
* ``bnn``, ``sbn``, ``hier`` -- the Bayesian-NN, sigmoid-belief-net and
                    ragged hierarchical families.

Parity status: TensorFlow 1.x (where the reference's arithmetic lives, pinned
``tensorflow==1.5.0`` in the reference's ``.travis.yml:40``) cannot be
installed here, so parity against the reference's own TF CPU path is
UNPINNED at the bit level.  The oracle is pinned instead to (a) the published
Philox4x32-10 known-answer vectors, (b) FP64 central finite differences of
every hand-written gradient and (c) the closed-form posteriors that the
reference's own tests assert (``tests/inferences/klqp_test.py:33-35``,
``tests/inferences/hmc_test.py:33-35,79-80``,
``tests/inferences/inference_auto_transform_test.py:187-188``).
"""
