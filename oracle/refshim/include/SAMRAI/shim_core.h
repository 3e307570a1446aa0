// Minimal stand-in for the part of SAMRAI (https://github.com/LLNL/SAMRAI, 4.x API) that the
// HAMeRS convective-flux translation units use on one patch.  Test infrastructure only: it lets
// the reference's own .cpp files compile unmodified, in place, so that their FP64 output can be
// compared with the oracle's.  Only what those files call is provided; every other SAMRAI
// service (hierarchies, schedules, MPI, restart, plotting) is absent.
//
// Layout follows SAMRAI's pdat arrays: one array per depth (component), x fastest, spanning the
// ghost box; a SideData array of axis a spans the ghost box grown by one cell at its upper end
// along a.
#ifndef HMR_REF_SAMRAI_SHIM_CORE_H
#define HMR_REF_SAMRAI_SHIM_CORE_H

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#define SAMRAI_SHARED_PTR_CAST std::dynamic_pointer_cast

// Errors become C++ exceptions; the shim's C entry point catches them and returns a status.
#define TBOX_ERROR(X)                                                       \
    do {                                                                    \
        std::ostringstream hmr_ref_os;                                      \
        hmr_ref_os << X;                                                    \
        throw std::runtime_error(hmr_ref_os.str());                         \
    } while (0)
#define TBOX_WARNING(X) do { } while (0)
// SAMRAI built without DEBUG_CHECK_ASSERTIONS (its release configuration): assertions compile
// to nothing, and their arguments are not compiled either.
#define TBOX_ASSERT(X) do { } while (0)
#define TBOX_DIM_ASSERT(X) do { } while (0)
#define NULL_STATEMENT do { } while (0)
#define TBOX_ASSERT_OBJDIM_EQUALITY2(a, b) do { } while (0)
#define TBOX_ASSERT_OBJDIM_EQUALITY3(a, b, c) do { } while (0)
#define TBOX_ASSERT_DIM_OBJDIM_EQUALITY1(d, a) do { } while (0)
#define NULL_USE(X) (void)(X)

namespace SAMRAI {

namespace tbox {

class Dimension {
public:
    explicit Dimension(unsigned short d) : d_(d) {}
    unsigned short getValue() const { return d_; }
    bool operator==(const Dimension& o) const { return d_ == o.d_; }
    bool operator!=(const Dimension& o) const { return d_ != o.d_; }
    bool operator<(const Dimension& o) const { return d_ < o.d_; }
    bool operator>(const Dimension& o) const { return d_ > o.d_; }
    bool operator<=(const Dimension& o) const { return d_ <= o.d_; }
    bool operator>=(const Dimension& o) const { return d_ >= o.d_; }
    static const int MAXIMUM_DIMENSION_VALUE = 3;

private:
    unsigned short d_;
};

inline std::ostream& pout_stream() { return std::cout; }
#define pout pout_stream()
#define plog pout_stream()
#define perr std::cerr

struct Utilities {
    static void abort(const std::string& m, const std::string&, int) { throw std::runtime_error(m); }
    static std::string intToString(int v, int = 1) { return std::to_string(v); }
    static std::string nodeToString(int v) { return std::to_string(v); }
    static std::string processorToString(int v) { return std::to_string(v); }
};

// One process: rank 0 of 1; reductions are identities.
class SAMRAI_MPI {
public:
    static const SAMRAI_MPI& getSAMRAIWorld() {
        static SAMRAI_MPI w;
        return w;
    }
    int getRank() const { return 0; }
    int getSize() const { return 1; }
    template <class T>
    int AllReduce(T*, int, int) const { return 0; }
    template <class T>
    int Allreduce(T*, T*, int, int, int) const { return 0; }
    int Barrier() const { return 0; }
};

template <class T>
struct MathUtilities {
    static T getMax() { return std::numeric_limits<T>::max(); }
    static T getMin() { return std::numeric_limits<T>::lowest(); }
    static T getEpsilon() { return std::numeric_limits<T>::epsilon(); }
    static T getSignalingNaN() { return std::numeric_limits<T>::signaling_NaN(); }
    static bool isNaN(const T& v) { return std::isnan(v); }
    static bool equalEps(const T& a, const T& b) {
        const T s = std::max(std::fabs(a), std::fabs(b));
        return std::fabs(a - b) <= 1.0e-12 * (s > 1.0 ? s : 1.0);
    }
    static T Max(T a, T b) { return a > b ? a : b; }
    static T Min(T a, T b) { return a < b ? a : b; }
    static T Abs(T a) { return a < 0 ? -a : a; }
};

// Key/value store with the typed getters the HAMeRS constructors read.
class Database {
public:
    explicit Database(const std::string& name = "db") : name_(name) {}
    virtual ~Database() {}
    const std::string& getName() const { return name_; }

    bool keyExists(const std::string& k) const {
        return d_.count(k) || s_.count(k) || i_.count(k) || b_.count(k) || db_.count(k);
    }
    std::vector<std::string> getAllKeys() const {
        std::vector<std::string> k;
        for (auto& p : d_) k.push_back(p.first);
        for (auto& p : s_) k.push_back(p.first);
        for (auto& p : i_) k.push_back(p.first);
        for (auto& p : b_) k.push_back(p.first);
        for (auto& p : db_) k.push_back(p.first);
        return k;
    }
    bool isDouble(const std::string& k) const { return d_.count(k) > 0; }
    bool isInteger(const std::string& k) const { return i_.count(k) > 0; }
    bool isString(const std::string& k) const { return s_.count(k) > 0; }
    bool isBool(const std::string& k) const { return b_.count(k) > 0; }
    bool isDatabase(const std::string& k) const { return db_.count(k) > 0; }
    size_t getArraySize(const std::string& k) const {
        if (d_.count(k)) return d_.at(k).size();
        if (i_.count(k)) return i_.at(k).size();
        if (s_.count(k)) return s_.at(k).size();
        if (b_.count(k)) return b_.at(k).size();
        return 0;
    }

    double getDouble(const std::string& k) const {
        if (d_.count(k)) return d_.at(k).at(0);
        if (i_.count(k)) return (double)i_.at(k).at(0);
        throw std::runtime_error("no double key " + k);
    }
    double getDoubleWithDefault(const std::string& k, double v) const { return keyExists(k) ? getDouble(k) : v; }
    float getFloat(const std::string& k) const { return (float)getDouble(k); }
    float getFloatWithDefault(const std::string& k, float v) const { return keyExists(k) ? getFloat(k) : v; }
    std::vector<double> getDoubleVector(const std::string& k) const {
        if (d_.count(k)) return d_.at(k);
        if (i_.count(k)) return std::vector<double>(i_.at(k).begin(), i_.at(k).end());
        throw std::runtime_error("no double vector key " + k);
    }
    void getDoubleArray(const std::string& k, double* out, size_t n) const {
        auto v = getDoubleVector(k);
        for (size_t i = 0; i < n && i < v.size(); i++) out[i] = v[i];
    }
    int getInteger(const std::string& k) const {
        if (i_.count(k)) return i_.at(k).at(0);
        throw std::runtime_error("no integer key " + k);
    }
    int getIntegerWithDefault(const std::string& k, int v) const { return keyExists(k) ? getInteger(k) : v; }
    std::vector<int> getIntegerVector(const std::string& k) const {
        if (i_.count(k)) return i_.at(k);
        throw std::runtime_error("no integer vector key " + k);
    }
    bool getBool(const std::string& k) const {
        if (b_.count(k)) return b_.at(k).at(0);
        throw std::runtime_error("no bool key " + k);
    }
    bool getBoolWithDefault(const std::string& k, bool v) const { return keyExists(k) ? getBool(k) : v; }
    std::vector<bool> getBoolVector(const std::string& k) const { return b_.at(k); }
    std::string getString(const std::string& k) const {
        if (s_.count(k)) return s_.at(k).at(0);
        throw std::runtime_error("no string key " + k);
    }
    std::string getStringWithDefault(const std::string& k, const std::string& v) const {
        return keyExists(k) ? getString(k) : v;
    }
    std::vector<std::string> getStringVector(const std::string& k) const { return s_.at(k); }
    std::shared_ptr<Database> getDatabase(const std::string& k) const {
        if (db_.count(k)) return db_.at(k);
        throw std::runtime_error("no database key " + k);
    }

    void getVector(const std::string& k, std::vector<double>& out) const { out = getDoubleVector(k); }
    void putVector(const std::string& k, const std::vector<double>& v) { d_[k] = v; }
    void putDouble(const std::string& k, double v) { d_[k] = {v}; }
    void putDoubleVector(const std::string& k, const std::vector<double>& v) { d_[k] = v; }
    void putDoubleArray(const std::string& k, const double* v, size_t n) { d_[k].assign(v, v + n); }
    void putInteger(const std::string& k, int v) { i_[k] = {v}; }
    void putIntegerVector(const std::string& k, const std::vector<int>& v) { i_[k] = v; }
    void putBool(const std::string& k, bool v) { b_[k] = {v}; }
    void putBoolVector(const std::string& k, const std::vector<bool>& v) { b_[k] = v; }
    void putString(const std::string& k, const std::string& v) { s_[k] = {v}; }
    void putStringVector(const std::string& k, const std::vector<std::string>& v) { s_[k] = v; }
    std::shared_ptr<Database> putDatabase(const std::string& k) {
        auto p = std::make_shared<Database>(k);
        db_[k] = p;
        return p;
    }

private:
    std::string name_;
    std::map<std::string, std::vector<double>> d_;
    std::map<std::string, std::vector<int>> i_;
    std::map<std::string, std::vector<bool>> b_;
    std::map<std::string, std::vector<std::string>> s_;
    std::map<std::string, std::shared_ptr<Database>> db_;
};

}  // namespace tbox

namespace hier {

class IntVector {
public:
    IntVector() : dim_(3) { v_[0] = v_[1] = v_[2] = 0; }
    explicit IntVector(const tbox::Dimension& d, int val = 0) : dim_(d.getValue()) {
        for (int i = 0; i < 3; i++) v_[i] = i < dim_ ? val : 0;
    }
    IntVector(const std::vector<int>& v, const tbox::Dimension& d) : dim_(d.getValue()) {
        for (int i = 0; i < 3; i++) v_[i] = i < dim_ ? v.at(i) : 0;
    }
    static const IntVector& getOne(const tbox::Dimension& d) { return table(d.getValue(), 1); }
    static const IntVector& getZero(const tbox::Dimension& d) { return table(d.getValue(), 0); }
    tbox::Dimension getDim() const { return tbox::Dimension((unsigned short)dim_); }
    int& operator[](int i) { return v_[i]; }
    const int& operator[](int i) const { return v_[i]; }
    int& operator()(int i) { return v_[i]; }
    const int& operator()(int i) const { return v_[i]; }
    long product() const {
        long p = 1;
        for (int i = 0; i < dim_; i++) p *= v_[i];
        return p;
    }
    int max() const {
        int m = v_[0];
        for (int i = 1; i < dim_; i++) m = std::max(m, v_[i]);
        return m;
    }
    int min() const {
        int m = v_[0];
        for (int i = 1; i < dim_; i++) m = std::min(m, v_[i]);
        return m;
    }
    static IntVector min(const IntVector& a, const IntVector& b) {
        IntVector r(a);
        for (int i = 0; i < r.dim_; i++) r.v_[i] = std::min(a.v_[i], b.v_[i]);
        return r;
    }
    static IntVector max(const IntVector& a, const IntVector& b) {
        IntVector r(a);
        for (int i = 0; i < r.dim_; i++) r.v_[i] = std::max(a.v_[i], b.v_[i]);
        return r;
    }
    void min(const IntVector& o) {
        for (int i = 0; i < dim_; i++) v_[i] = std::min(v_[i], o.v_[i]);
    }
    void max(const IntVector& o) {
        for (int i = 0; i < dim_; i++) v_[i] = std::max(v_[i], o.v_[i]);
    }
#define HMR_REF_IV_OP(op)                                                   \
    IntVector operator op(const IntVector& o) const {                       \
        IntVector r(*this);                                                 \
        for (int i = 0; i < dim_; i++) r.v_[i] = v_[i] op o.v_[i];          \
        return r;                                                           \
    }                                                                       \
    IntVector operator op(int s) const {                                    \
        IntVector r(*this);                                                 \
        for (int i = 0; i < dim_; i++) r.v_[i] = v_[i] op s;                \
        return r;                                                           \
    }                                                                       \
    IntVector& operator op##=(const IntVector& o) {                         \
        for (int i = 0; i < dim_; i++) v_[i] = v_[i] op o.v_[i];            \
        return *this;                                                       \
    }                                                                       \
    IntVector& operator op##=(int s) {                                      \
        for (int i = 0; i < dim_; i++) v_[i] = v_[i] op s;                  \
        return *this;                                                       \
    }
    HMR_REF_IV_OP(+)
    HMR_REF_IV_OP(-)
    HMR_REF_IV_OP(*)
    HMR_REF_IV_OP(/)
#undef HMR_REF_IV_OP
    IntVector operator-() const {
        IntVector r(*this);
        for (int i = 0; i < dim_; i++) r.v_[i] = -v_[i];
        return r;
    }
    bool operator==(const IntVector& o) const {
        for (int i = 0; i < dim_; i++)
            if (v_[i] != o.v_[i]) return false;
        return true;
    }
    bool operator!=(const IntVector& o) const { return !(*this == o); }
    bool operator==(int s) const {
        for (int i = 0; i < dim_; i++)
            if (v_[i] != s) return false;
        return true;
    }
    bool operator!=(int s) const { return !(*this == s); }
#define HMR_REF_IV_CMP(op)                                                  \
    bool operator op(const IntVector& o) const {                            \
        for (int i = 0; i < dim_; i++)                                      \
            if (!(v_[i] op o.v_[i])) return false;                          \
        return true;                                                        \
    }                                                                       \
    bool operator op(int s) const {                                         \
        for (int i = 0; i < dim_; i++)                                      \
            if (!(v_[i] op s)) return false;                                \
        return true;                                                        \
    }
    HMR_REF_IV_CMP(<)
    HMR_REF_IV_CMP(<=)
    HMR_REF_IV_CMP(>)
    HMR_REF_IV_CMP(>=)
#undef HMR_REF_IV_CMP
    int getDimVal() const { return dim_; }

private:
    static const IntVector& table(int d, int val) {
        static IntVector t[4][2] = {
            {IntVector(tbox::Dimension(1), 0), IntVector(tbox::Dimension(1), 1)},
            {IntVector(tbox::Dimension(1), 0), IntVector(tbox::Dimension(1), 1)},
            {IntVector(tbox::Dimension(2), 0), IntVector(tbox::Dimension(2), 1)},
            {IntVector(tbox::Dimension(3), 0), IntVector(tbox::Dimension(3), 1)}};
        return t[d][val];
    }
    int dim_;
    int v_[3];
};

inline std::ostream& operator<<(std::ostream& os, const IntVector& v) {
    os << "(";
    for (int i = 0; i < v.getDimVal(); i++) os << (i ? "," : "") << v[i];
    return os << ")";
}

class Index : public IntVector {
public:
    Index() : IntVector() {}
    explicit Index(const tbox::Dimension& d, int val = 0) : IntVector(d, val) {}
    Index(const IntVector& v) : IntVector(v) {}
};

class BlockId {
public:
    explicit BlockId(int v = 0) : v_(v) {}
    int getBlockValue() const { return v_; }

private:
    int v_;
};

class Box {
public:
    explicit Box(const tbox::Dimension& d) : lo_(d, 0), hi_(d, -1) {}
    Box(const IntVector& lo, const IntVector& hi, const BlockId& = BlockId(0)) : lo_(lo), hi_(hi) {}
    static Box getEmptyBox(const tbox::Dimension& d) { return Box(d); }
    tbox::Dimension getDim() const { return lo_.getDim(); }
    Index& lower() { return lo_; }
    Index& upper() { return hi_; }
    const Index& lower() const { return lo_; }
    const Index& upper() const { return hi_; }
    int lower(int d) const { return lo_[d]; }
    int upper(int d) const { return hi_[d]; }
    void setLower(const IntVector& v) { lo_ = v; }
    void setUpper(const IntVector& v) { hi_ = v; }
    bool empty() const {
        for (int i = 0; i < lo_.getDimVal(); i++)
            if (hi_[i] < lo_[i]) return true;
        return false;
    }
    IntVector numberCells() const {
        if (empty()) return IntVector::getZero(getDim());
        return hi_ - lo_ + 1;
    }
    int numberCells(int d) const { return empty() ? 0 : hi_[d] - lo_[d] + 1; }
    long size() const { return numberCells().product(); }
    Box& grow(const IntVector& g) {
        if (!empty()) {
            lo_ -= g;
            hi_ += g;
        }
        return *this;
    }
    Box& grow(int d, int g) {
        if (!empty()) {
            lo_[d] -= g;
            hi_[d] += g;
        }
        return *this;
    }
    Box& growUpper(int d, int g) {
        hi_[d] += g;
        return *this;
    }
    Box& shift(const IntVector& s) {
        lo_ += s;
        hi_ += s;
        return *this;
    }
    bool contains(const Box& b) const {
        if (b.empty()) return true;
        return b.lo_ >= lo_ && b.hi_ <= hi_;
    }
    bool contains(const IntVector& p) const { return p >= lo_ && p <= hi_; }
    Box operator*(const Box& o) const {
        Box r(*this);
        for (int i = 0; i < lo_.getDimVal(); i++) {
            r.lo_[i] = std::max(lo_[i], o.lo_[i]);
            r.hi_[i] = std::min(hi_[i], o.hi_[i]);
        }
        return r;
    }
    bool operator==(const Box& o) const { return lo_ == o.lo_ && hi_ == o.hi_; }
    bool isSpatiallyEqual(const Box& o) const { return *this == o || (empty() && o.empty()); }
    bool operator!=(const Box& o) const { return !(*this == o); }
    long offset(const IntVector& p) const {
        const IntVector n = numberCells();
        long o = 0, s = 1;
        for (int i = 0; i < lo_.getDimVal(); i++) {
            o += (long)(p[i] - lo_[i]) * s;
            s *= n[i];
        }
        return o;
    }

private:
    Index lo_, hi_;
};

inline std::ostream& operator<<(std::ostream& os, const Box& b) {
    return os << "[" << b.lower() << "," << b.upper() << "]";
}

class VariableContext {
public:
    explicit VariableContext(const std::string& n) : name_(n) {}
    const std::string& getName() const { return name_; }

private:
    std::string name_;
};

class Variable {
public:
    Variable(const tbox::Dimension& d, const std::string& n) : dim_(d), name_(n) {}
    virtual ~Variable() {}
    const std::string& getName() const { return name_; }
    const tbox::Dimension& getDim() const { return dim_; }

private:
    tbox::Dimension dim_;
    std::string name_;
};

class PatchData {
public:
    PatchData(const Box& box, const IntVector& ghosts)
        : box_(box), ghost_box_(Box(box).grow(ghosts)), ghosts_(ghosts) {}
    virtual ~PatchData() {}
    const Box& getBox() const { return box_; }
    const Box& getGhostBox() const { return ghost_box_; }
    const IntVector& getGhostCellWidth() const { return ghosts_; }
    tbox::Dimension getDim() const { return box_.getDim(); }
    double getTime() const { return time_; }
    void setTime(double t) { time_ = t; }

protected:
    Box box_;
    Box ghost_box_;
    IntVector ghosts_;
    double time_ = 0.0;
};

class PatchGeometry {
public:
    virtual ~PatchGeometry() {}
};

// A boundary box: the one-cell-thick box of ghost cells beside a patch side, edge or corner
// that lies on the physical boundary, with its codimension (SAMRAI's boundary type) and its
// location index (the BDRY_LOC / NODE_BDRY_LOC_2D / EDGE_BDRY_LOC_3D / NODE_BDRY_LOC_3D
// numbering of CartesianBoundaryDefines.hpp).
class BoundaryBox {
public:
    BoundaryBox() : box_(tbox::Dimension(1)) {}
    BoundaryBox(const Box& box, int type, int loc) : box_(box), type_(type), loc_(loc) {}
    const Box& getBox() const { return box_; }
    int getBoundaryType() const { return type_; }
    int getLocationIndex() const { return loc_; }

private:
    Box box_;
    int type_ = 0;
    int loc_ = 0;
};

// Types that appear only in declarations of services this build does not provide
// (hierarchies, levels).
class PatchHierarchy {};
class PatchLevel {};

// A patch: its interior box, its geometry and the data registered on it by
// (variable, context).
class Patch {
public:
    Patch(const Box& box, const std::shared_ptr<PatchGeometry>& geom) : box_(box), geom_(geom) {}
    const Box& getBox() const { return box_; }
    tbox::Dimension getDim() const { return box_.getDim(); }
    const std::shared_ptr<PatchGeometry>& getPatchGeometry() const { return geom_; }
    std::shared_ptr<PatchData> getPatchData(const std::shared_ptr<Variable>& v,
                                            const std::shared_ptr<VariableContext>& c) const {
        auto it = data_.find(key(v.get(), c.get()));
        if (it == data_.end())
            throw std::runtime_error("no patch data for variable " + v->getName() + " in context " + c->getName());
        return it->second;
    }
    void setPatchData(const std::shared_ptr<Variable>& v, const std::shared_ptr<VariableContext>& c,
                      const std::shared_ptr<PatchData>& d) {
        data_[key(v.get(), c.get())] = d;
    }
    int getPatchLevelNumber() const { return 0; }

private:
    static std::pair<const void*, const void*> key(const void* v, const void* c) { return {v, c}; }
    Box box_;
    std::shared_ptr<PatchGeometry> geom_;
    std::map<std::pair<const void*, const void*>, std::shared_ptr<PatchData>> data_;
};

// Registry of (variable, context) pairs; the flow models register their conservative
// variables here.  Index lookups are not needed on one patch.
class VariableDatabase {
public:
    static VariableDatabase* getDatabase() {
        static VariableDatabase db;
        return &db;
    }
    std::shared_ptr<VariableContext> getContext(const std::string& name) {
        auto& c = contexts_[name];
        if (!c) c = std::make_shared<VariableContext>(name);
        return c;
    }
    int registerVariableAndContext(const std::shared_ptr<Variable>&, const std::shared_ptr<VariableContext>&,
                                   const IntVector& = IntVector()) {
        return next_++;
    }
    int mapVariableAndContextToIndex(const std::shared_ptr<Variable>&, const std::shared_ptr<VariableContext>&) {
        return -1;
    }

private:
    std::map<std::string, std::shared_ptr<VariableContext>> contexts_;
    int next_ = 0;
};

}  // namespace hier

namespace pdat {

// Sets v on the cells of `region` inside `array_box`, in an array laid out over array_box.
template <class T>
void fill_region(T* p, const hier::Box& array_box, const hier::Box& region, const T& v) {
    const hier::Box r = region * array_box;
    if (r.empty()) return;
    const int dim = array_box.getDim().getValue();
    hier::IntVector i(r.lower());
    for (;;) {
        p[array_box.offset(i)] = v;
        int a = 0;
        while (a < dim) {
            if (++i[a] <= r.upper()[a]) break;
            i[a] = r.lower()[a];
            a++;
        }
        if (a == dim) break;
    }
}

template <class T>
class CellData : public hier::PatchData {
public:
    CellData(const hier::Box& box, int depth, const hier::IntVector& ghosts)
        : hier::PatchData(box, ghosts), depth_(depth),
          n_(ghost_box_.size()), data_((size_t)depth * (size_t)ghost_box_.size()) {}
    int getDepth() const { return depth_; }
    T* getPointer(int d = 0) { return data_.data() + (size_t)d * n_; }
    const T* getPointer(int d = 0) const { return data_.data() + (size_t)d * n_; }
    void fill(const T& v, int d = 0) { std::fill(getPointer(d), getPointer(d) + n_, v); }
    void fill(const T& v, const hier::Box& region, int d = 0) { fill_region(getPointer(d), ghost_box_, region, v); }
    void fillAll(const T& v) { std::fill(data_.begin(), data_.end(), v); }
    void fillAll(const T& v, const hier::Box& region) {
        for (int d = 0; d < depth_; d++) fill(v, region, d);
    }
    long getArraySize() const { return n_; }
    // Copies depth `src_depth` of `src` into depth `dst_depth` over the common ghost box.
    void copyDepth(int dst_depth, const CellData<T>& src, int src_depth) {
        const hier::Box r = ghost_box_ * src.getGhostBox();
        if (r.empty()) return;
        const int dim = box_.getDim().getValue();
        hier::IntVector i(r.lower());
        for (;;) {
            getPointer(dst_depth)[ghost_box_.offset(i)] = src.getPointer(src_depth)[src.getGhostBox().offset(i)];
            int a = 0;
            while (a < dim) {
                if (++i[a] <= r.upper()[a]) break;
                i[a] = r.lower()[a];
                a++;
            }
            if (a == dim) break;
        }
    }

private:
    int depth_;
    long n_;
    std::vector<T> data_;
};

template <class T>
class SideData : public hier::PatchData {
public:
    SideData(const hier::Box& box, int depth, const hier::IntVector& ghosts)
        : SideData(box, depth, ghosts, hier::IntVector::getOne(box.getDim())) {}
    SideData(const hier::Box& box, int depth, const hier::IntVector& ghosts, const hier::IntVector& directions)
        : hier::PatchData(box, ghosts), depth_(depth), dirs_(directions) {
        const int dim = box.getDim().getValue();
        for (int a = 0; a < dim; a++) {
            hier::Box sb(ghost_box_);
            sb.growUpper(a, 1);
            side_boxes_.push_back(sb);
            n_.push_back(sb.size());
            arrays_.emplace_back(dirs_[a] ? (size_t)depth * (size_t)sb.size() : 0);
        }
    }
    int getDepth() const { return depth_; }
    const hier::IntVector& getDirectionVector() const { return dirs_; }
    T* getPointer(int axis, int d = 0) { return arrays_.at(axis).data() + (size_t)d * n_[axis]; }
    const T* getPointer(int axis, int d = 0) const { return arrays_.at(axis).data() + (size_t)d * n_[axis]; }
    void fill(const T& v, int d = 0) {
        for (size_t a = 0; a < arrays_.size(); a++)
            if (!arrays_[a].empty()) std::fill(getPointer((int)a, d), getPointer((int)a, d) + n_[a], v);
    }
    void fillAll(const T& v) {
        for (auto& a : arrays_) std::fill(a.begin(), a.end(), v);
    }
    // Sides of the cells of `region`: along axis a, the region grown by one at its upper end.
    void fill(const T& v, const hier::Box& region, int d = 0) {
        for (size_t a = 0; a < arrays_.size(); a++) {
            if (arrays_[a].empty()) continue;
            hier::Box r(region);
            r.growUpper((int)a, 1);
            fill_region(getPointer((int)a, d), side_boxes_[a], r, v);
        }
    }
    void fillAll(const T& v, const hier::Box& region) {
        for (int d = 0; d < depth_; d++) fill(v, region, d);
    }
    const hier::Box& getSideBox(int axis) const { return side_boxes_.at(axis); }

private:
    int depth_;
    hier::IntVector dirs_;
    std::vector<hier::Box> side_boxes_;
    std::vector<long> n_;
    std::vector<std::vector<T>> arrays_;
};

template <class T>
class CellVariable : public hier::Variable {
public:
    CellVariable(const tbox::Dimension& d, const std::string& n, int depth = 1)
        : hier::Variable(d, n), depth_(depth) {}
    int getDepth() const { return depth_; }

private:
    int depth_;
};

template <class T>
class SideVariable : public hier::Variable {
public:
    SideVariable(const tbox::Dimension& d, const std::string& n, int depth = 1)
        : hier::Variable(d, n), depth_(depth) {}
    SideVariable(const tbox::Dimension& d, const std::string& n, const hier::IntVector&, int depth = 1)
        : hier::Variable(d, n), depth_(depth) {}
    int getDepth() const { return depth_; }

private:
    int depth_;
};

}  // namespace pdat

namespace geom {

class CartesianGridGeometry {
public:
    CartesianGridGeometry(const tbox::Dimension& d, const double* dx, const double* xlo) : dim_(d) {
        for (int i = 0; i < 3; i++) {
            dx_[i] = i < d.getValue() ? dx[i] : 1.0;
            xlo_[i] = xlo ? xlo[i] : 0.0;
        }
    }
    const double* getDx() const { return dx_; }
    const double* getXLower() const { return xlo_; }
    const tbox::Dimension& getDim() const { return dim_; }

private:
    tbox::Dimension dim_;
    double dx_[3];
    double xlo_[3];
};

class CartesianPatchGeometry : public hier::PatchGeometry {
public:
    CartesianPatchGeometry(const double* dx, const double* xlo) {
        for (int i = 0; i < 3; i++) {
            dx_[i] = dx[i];
            xlo_[i] = xlo ? xlo[i] : 0.0;
        }
    }
    const double* getDx() const { return dx_; }
    const double* getXLower() const { return xlo_; }
    // Boundary boxes of the patch by codimension (1..3); none unless a caller sets them, so a
    // patch touches no physical boundary by default.
    void setCodimensionBoundaries(int codim, const std::vector<hier::BoundaryBox>& boxes) { bdry_[codim] = boxes; }
    std::vector<hier::BoundaryBox> getCodimensionBoundaries(int codim) const {
        return codim >= 1 && codim <= 3 ? bdry_[codim] : std::vector<hier::BoundaryBox>();
    }
    // The ghost cells a boundary box stands for: along each axis on which the box lies
    // outside the patch, the `gcw` cells beyond that side; along the others the box's own
    // extent.  Empty where gcw is 0 along an outward axis.
    hier::Box getBoundaryFillBox(const hier::BoundaryBox& bb, const hier::Box& b, const hier::IntVector& gcw) const {
        hier::Box f = bb.getBox();
        for (int d = 0; d < b.getDim().getValue(); d++) {
            if (f.upper(d) < b.lower(d)) {
                if (gcw[d] <= 0) return hier::Box::getEmptyBox(b.getDim());
                f.lower()[d] = b.lower(d) - gcw[d];
                f.upper()[d] = b.lower(d) - 1;
            } else if (f.lower(d) > b.upper(d)) {
                if (gcw[d] <= 0) return hier::Box::getEmptyBox(b.getDim());
                f.lower()[d] = b.upper(d) + 1;
                f.upper()[d] = b.upper(d) + gcw[d];
            }
        }
        return f;
    }

private:
    double dx_[3];
    double xlo_[3];
    std::vector<hier::BoundaryBox> bdry_[4];
};

}  // namespace geom

namespace appu {

class VisDerivedDataStrategy {
public:
    virtual ~VisDerivedDataStrategy() {}
};

class VisItDataWriter {};

}  // namespace appu

}  // namespace SAMRAI

#endif  // HMR_REF_SAMRAI_SHIM_CORE_H
