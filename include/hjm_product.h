/*
 * hjm_product.h -- the product types of the drop-in entry points.
 *
 * Layout- and constructor-compatible with the reference's InterestRateSwap
 * (mahsanchez/cva_hjm_cuda product.h:4-18): three schedule pointers (never
 * read by any computation, there or here), notional, fixed rate K, accrual
 * period dtau and expiry, in that member order; and with its double-only
 * twin InterestRateSwap_D (product.h:20-34), which the reference's driver
 * constructs (simulation_gpu_testing.cpp:216) though no entry point takes it.
 * It uses the reference header's include guard, so whichever of the two
 * headers a translation unit includes first provides both types and the
 * other is skipped: the reference's driver compiles unchanged against this
 * library.
 */
#ifndef INTEREST_RATE_SWAP
#define INTEREST_RATE_SWAP

template <typename real>
struct InterestRateSwap {
    InterestRateSwap(real* pricing_points_, real* floating_schedule_, real* fixed_schedule_, real notional_,
                     real K_, real expiry_, real dtau_)
        : pricing_points(pricing_points_),
          realing_schedule(floating_schedule_),
          fixed_schedule(fixed_schedule_),
          notional(notional_),
          K(K_),
          dtau(dtau_),
          expiry(expiry_)
    {
    }

    real* pricing_points;
    real* realing_schedule; /* the floating-leg schedule; member name kept for source compatibility */
    real* fixed_schedule;
    real notional;
    real K;
    real dtau;
    real expiry;
};

/* The double-precision swap as a plain struct (same members, same order, same
 * constructor argument order: ..., notional, K, expiry, dtau). */
struct InterestRateSwap_D {
    InterestRateSwap_D(double* pricing_points_, double* floating_schedule_, double* fixed_schedule_,
                       double notional_, double K_, double expiry_, double dtau_)
        : pricing_points(pricing_points_),
          realing_schedule(floating_schedule_),
          fixed_schedule(fixed_schedule_),
          notional(notional_),
          K(K_),
          dtau(dtau_),
          expiry(expiry_)
    {
    }

    double* pricing_points;
    double* realing_schedule;
    double* fixed_schedule;
    double notional;
    double K;
    double dtau;
    double expiry;
};

#endif
