/*
 * hjm_product.h -- the product type of the drop-in entry points.
 *
 * Layout- and constructor-compatible with the reference's InterestRateSwap
 * (mahsanchez/cva_hjm_cuda product.h:4-18): three schedule pointers (never
 * read by any computation, there or here), notional, fixed rate K, accrual
 * period dtau and expiry, in that member order.  It uses the reference
 * header's include guard so that a program that already includes the
 * reference's product.h sees one definition.
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

#endif
