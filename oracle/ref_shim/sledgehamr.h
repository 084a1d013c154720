/* ORACLE (test infrastructure only).
 *
 * Stand-in for source/sledgehamr.h when only the projects' kernel headers
 * are compiled for oracle/_ref: it defines the field and hook macros of
 * source/macros.h:39-181 without Boost.Preprocessor (supports up to eight
 * names per macro, enough for every project), and includes the reference's
 * own kernels.h and sledgehamr_utils.h from the include path.
 */
#ifndef SH_REF_SHIM_SLEDGEHAMR_H_
#define SH_REF_SHIM_SLEDGEHAMR_H_

#include <kernels.h>
#include <sledgehamr_utils.h>

namespace sledgehamr {
struct ScalarField {
    ScalarField(std::string s, std::vector<ScalarField *> &v, bool m)
        : name(s), id((int)v.size()), is_conjugate_momentum(m) { v.push_back(this); }
    operator int() const { return id; }
    std::string name;
    const int id;
    bool is_conjugate_momentum;
};
} // namespace sledgehamr

#define RS_CAT(a, b) RS_CAT_I(a, b)
#define RS_CAT_I(a, b) a##b
#define RS_NARG(...) RS_NARG_I(__VA_ARGS__, 8, 7, 6, 5, 4, 3, 2, 1, 0)
#define RS_NARG_I(_1, _2, _3, _4, _5, _6, _7, _8, N, ...) N
#define RS_EACH(M, ...) RS_CAT(RS_E_, RS_NARG(__VA_ARGS__))(M, __VA_ARGS__)
#define RS_E_1(M, a) M(a)
#define RS_E_2(M, a, ...) M(a) RS_E_1(M, __VA_ARGS__)
#define RS_E_3(M, a, ...) M(a) RS_E_2(M, __VA_ARGS__)
#define RS_E_4(M, a, ...) M(a) RS_E_3(M, __VA_ARGS__)
#define RS_E_5(M, a, ...) M(a) RS_E_4(M, __VA_ARGS__)
#define RS_E_6(M, a, ...) M(a) RS_E_5(M, __VA_ARGS__)
#define RS_E_7(M, a, ...) M(a) RS_E_6(M, __VA_ARGS__)
#define RS_E_8(M, a, ...) M(a) RS_E_7(M, __VA_ARGS__)

#define RS_ENUM_ENTRY(f) f,
#define RS_ONE_SCALAR(f)                                                       \
    static sledgehamr::ScalarField RS_CAT(_s_, f) = {#f, l_scalar_fields, false}; \
    namespace Scalar { constexpr int f = _Scalar::f; }
#define RS_ONE_MOMENTUM(f)                                                     \
    static sledgehamr::ScalarField RS_CAT(_s_, f) = {#f, l_scalar_fields, true};  \
    namespace Scalar { constexpr int f = _Momentum::f + _Scalar::NScalarFields; }

#define SLEDGEHAMR_ADD_SCALARS(...)                                            \
    enum _Scalar { RS_EACH(RS_ENUM_ENTRY, __VA_ARGS__) NScalarFields };        \
    static std::vector<sledgehamr::ScalarField *> l_scalar_fields;             \
    RS_EACH(RS_ONE_SCALAR, __VA_ARGS__)

#define SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(...)                                  \
    enum _Momentum { RS_EACH(RS_ENUM_ENTRY, __VA_ARGS__) NMomentumFields };    \
    RS_EACH(RS_ONE_MOMENTUM, __VA_ARGS__)                                      \
    namespace Scalar {                                                         \
    constexpr int NScalars = _Scalar::NScalarFields + _Momentum::NMomentumFields; \
    }                                                                          \
    enum Gw { u_xx = Scalar::NScalars, u_yy, u_zz, u_xy, u_xz, u_yz,           \
              du_xx, du_yy, du_zz, du_xy, du_xz, du_yz, NGwScalars };          \
    template <int> inline double TruncationModifier(                           \
        const amrex::Array4<const double> &, const int, const int, const int,  \
        const int, const double, const double, const double, const double te,  \
        const double *) { return te; }                                         \
    template <bool> inline bool TagCellForRefinement(                          \
        const amrex::Array4<const double> &, const int, const int, const int,  \
        const int, const double, const double, const double, const double *) { \
        return false; }                                                        \
    template <bool> inline void GravitationalWavesRhs(                         \
        const amrex::Array4<double> &, const amrex::Array4<const double> &,    \
        const int, const int, const int, const int, const double, const double,\
        const double, const double *) {}                                       \
    template <bool> inline void GravitationalWavesBackreaction(                \
        const amrex::Array4<double> &, const amrex::Array4<const double> &,    \
        const int, const int, const int, const int, const double, const double,\
        const double, const double *, const double *) {}

#define SLEDGEHAMR_FINISH_SETUP

namespace sledgehamr {
/* Host-side project base class, enough for the project headers that define
 * their class next to their kernels (MinimalExample.h). */
class Sledgehamr {
  public:
    virtual ~Sledgehamr() = default;
    virtual void Init() {}
    virtual void SetParamsRhs(std::vector<double> &, const double, const int) {}
    std::vector<ScalarField *> scalar_fields;
};
} // namespace sledgehamr
#define SLEDGEHAMR_INITIALIZE_PROJECT(prj) prj() { scalar_fields = l_scalar_fields; }

#endif // SH_REF_SHIM_SLEDGEHAMR_H_
