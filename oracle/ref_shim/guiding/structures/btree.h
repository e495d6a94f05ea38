// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// Stand-in for libguiding's BTree (an empty submodule in the reference), enough for
// PathTracer (path.h:17-138) to compile and run with doGuiding = false: the plain method
// never samples, trains or steps the tree. Every member the wrapper touches exists; the
// distribution is uniform over [0,1)^2 (pdf 1, sample leaves the point unchanged), so a
// guided run through this stub would be the unguided estimator, and is not used.
#pragma once
#include <hussar/core/guiding.h>

namespace guiding {

struct Empty {};

template <typename T> struct Leaf {
    struct Settings {
        bool secondMoment = false;
    };
};

template <int D, typename L, typename A, template <typename> class Alloc> class BTree {
public:
    typedef VectorXf<D> Vector;
    typedef A AuxWrapper;
    struct Settings {
        Float splitThreshold = 0.f;
        typename L::Settings child;
    };

    template <typename... Args> Float pdf(const Settings &, const Vector &, Args &&...) const { return 1.f; }
    template <typename... Args> void sample(const Settings &, Float &pdf, Vector &, Args &&...) const { pdf = 1.f; }
    template <typename... Args> void splat(const Settings &, Float, const AuxWrapper &, Float, Args &&...) {}
    void build(const Settings &) {}
    void refine(const Settings &) {}
};

}  // namespace guiding
