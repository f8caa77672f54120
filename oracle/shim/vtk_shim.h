// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Minimal stand-in for the VTK >= 9.0 classes that the reference's clustering
// headers use (VTK is not installed here and cannot be).  Only the members the
// hot path touches exist; numerics come from oracle/restated_math.h.  The
// reference's own headers (Common/vtkUniformClustering.h,
// DiscreteRemeshing/vtkSurfaceClustering.h, vtkVerticesProcessing.h, the three
// metric headers) and Common/vtkQuadricTools.cxx are compiled UNMODIFIED
// against this directory by oracle/Makefile; shim/preinclude.h makes the shim
// vtkSurface and RenderWindow replace the reference's VTK-bound ones.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <queue>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../restated_math.h"

using std::cout;
using std::endl;
using std::setprecision;

typedef long long vtkIdType;

#define VTK_EXPORT
#define VTK_THREAD_RETURN_TYPE void*
#define VTK_THREAD_RETURN_VALUE nullptr
#define VTK_TRIANGLE 5
#define VTK_QUAD 9
#define VTK_POLYGON 7
#define VTK_MAJOR_VERSION 9
#define VTK_MINOR_VERSION 4

#define vtkSetMacro(name, type) \
    virtual void Set##name(type _arg) { this->name = _arg; }
#define vtkGetMacro(name, type) \
    virtual type Get##name() { return this->name; }
#define vtkStandardNewMacro(thisClass) \
    thisClass* thisClass::New() { return new thisClass; }
#define vtkTypeMacro(thisClass, superClass) typedef superClass Superclass;
#define vtkGetObjectMacro(name, type) \
    virtual type* Get##name() { return this->name; }
#define vtkGenericWarningMacro(x) \
    do { std::cerr << "warning: " << x << std::endl; } while (0)
#define VTK_LINE 3

class vtkObjectBase {
public:
    virtual ~vtkObjectBase() {}
    void Register(vtkObjectBase*) { ++RefCount; }
    void UnRegister(vtkObjectBase*) { if (--RefCount <= 0) delete this; }
    void Delete() { UnRegister(nullptr); }
protected:
    int RefCount = 1;
};

class vtkObject : public vtkObjectBase {
public:
    static vtkObject* New() { return new vtkObject; }
    virtual void Modified() {}
};

class vtkObjectFactory {
public:
    static vtkObject* CreateInstance(const char*) { return nullptr; }
};

class vtkCommand {};

class vtkIdList : public vtkObject {
public:
    static vtkIdList* New() { return new vtkIdList; }
    vtkIdType GetNumberOfIds() const { return (vtkIdType)Ids.size(); }
    vtkIdType GetId(vtkIdType i) const { return Ids[i]; }
    void SetId(vtkIdType i, vtkIdType v) { Ids[i] = v; }
    void SetNumberOfIds(vtkIdType n) { Ids.resize(n); }
    void Allocate(vtkIdType n) { Ids.reserve(n); }
    vtkIdType InsertNextId(vtkIdType v) { Ids.push_back(v); return (vtkIdType)Ids.size() - 1; }
    vtkIdType InsertUniqueId(vtkIdType v) {
        for (size_t i = 0; i < Ids.size(); i++) if (Ids[i] == v) return (vtkIdType)i;
        return InsertNextId(v);
    }
    vtkIdType IsId(vtkIdType v) const {
        for (size_t i = 0; i < Ids.size(); i++) if (Ids[i] == v) return (vtkIdType)i;
        return -1;
    }
    // removes every occurrence; the last entry takes the freed slot
    void DeleteId(vtkIdType v) {
        size_t i = 0;
        while (i < Ids.size()) {
            if (Ids[i] == v) { Ids[i] = Ids.back(); Ids.pop_back(); }
            else i++;
        }
    }
    void Reset() { Ids.clear(); }
    void Initialize() { Ids.clear(); }
    vtkIdType* GetPointer(vtkIdType i) { return Ids.data() + i; }
private:
    std::vector<vtkIdType> Ids;
};

class vtkDataArray : public vtkObject {
public:
    virtual double GetTuple1(vtkIdType i) = 0;
};

template <class T>
class vtkShimArray : public vtkDataArray {
public:
    void SetNumberOfValues(vtkIdType n) { V.resize(n); }
    void SetNumberOfComponents(int c) { NumComp = c; }
    int GetNumberOfComponents() const { return NumComp; }
    void SetNumberOfTuples(vtkIdType n) { V.resize(n * NumComp); }
    vtkIdType GetNumberOfTuples() const { return (vtkIdType)V.size() / NumComp; }
    vtkIdType GetNumberOfValues() const { return (vtkIdType)V.size(); }
    vtkIdType GetSize() const { return (vtkIdType)V.size(); }
    T GetValue(vtkIdType i) const { return V[i]; }
    void SetValue(vtkIdType i, T v) { V[i] = v; }
    vtkIdType InsertNextValue(T v) { V.push_back(v); return (vtkIdType)V.size() - 1; }
    T* GetPointer(vtkIdType i) { return V.data() + i; }
    double GetTuple1(vtkIdType i) override { return (double)V[i]; }
    void GetRange(double r[2]) {
        r[0] = 1e300; r[1] = -1e300;
        for (T x : V) { r[0] = std::min(r[0], (double)x); r[1] = std::max(r[1], (double)x); }
    }
    std::vector<T> V;
    int NumComp = 1;
};

class vtkIntArray : public vtkShimArray<int> {
public:
    static vtkIntArray* New() { return new vtkIntArray; }
};
class vtkDoubleArray : public vtkShimArray<double> {
public:
    static vtkDoubleArray* New() { return new vtkDoubleArray; }
};
class vtkFloatArray : public vtkShimArray<float> {
public:
    static vtkFloatArray* New() { return new vtkFloatArray; }
};
class vtkIdTypeArray : public vtkShimArray<vtkIdType> {
public:
    static vtkIdTypeArray* New() { return new vtkIdTypeArray; }
};
class vtkBitArray : public vtkShimArray<unsigned char> {
public:
    static vtkBitArray* New() { return new vtkBitArray; }
    int GetValue(vtkIdType i) const { return V[i] ? 1 : 0; }
    void SetValue(vtkIdType i, int v) { V[i] = v ? 1 : 0; }
};

class vtkDataArrayCollection : public vtkObject {
public:
    static vtkDataArrayCollection* New() { return new vtkDataArrayCollection; }
    ~vtkDataArrayCollection() override { for (auto* a : Items) a->UnRegister(this); }
    void AddItem(vtkDataArray* a) { a->Register(this); Items.push_back(a); }
    vtkDataArray* GetItem(int i) { return Items[i]; }
    void ReplaceItem(int i, vtkDataArray* a) { a->Register(this); Items[i]->UnRegister(this); Items[i] = a; }
    int GetNumberOfItems() const { return (int)Items.size(); }
private:
    std::vector<vtkDataArray*> Items;
};

class vtkTimerLog : public vtkObject {
public:
    static vtkTimerLog* New() { return new vtkTimerLog; }
    static double GetUniversalTime() {
        return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }
    void StartTimer() { T0 = GetUniversalTime(); }
    void StopTimer() { T1 = GetUniversalTime(); }
    double GetElapsedTime() { return T1 - T0; }
private:
    double T0 = 0, T1 = 0;
};

class vtkMath : public vtkObject {
public:
    static vtkMath* New() { return new vtkMath; }
    static double Dot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
    static double Distance2BetweenPoints(const double a[3], const double b[3]) { return rmath::dist2(a, b); }
    static void Cross(const double a[3], const double b[3], double c[3]) {
        const double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
        c[0] = x; c[1] = y; c[2] = z;
    }
    static double Norm(const double a[3]) { return std::sqrt(Dot(a, a)); }
    static double Normalize(double a[3]) {
        const double n = Norm(a);
        if (n != 0.0) { a[0] /= n; a[1] /= n; a[2] /= n; }
        return n;
    }
    static void Multiply3x3(const double A[3][3], const double in[3], double out[3]) { rmath::mul33v(A, in, out); }
    static void Multiply3x3(const double A[3][3], const double B[3][3], double C[3][3]) { rmath::mul33(A, B, C); }
    static void Transpose3x3(const double A[3][3], double AT[3][3]) { rmath::transpose33(A, AT); }
    static void SingularValueDecomposition3x3(const double A[3][3], double U[3][3], double w[3], double VT[3][3]) {
        rmath::svd3(A, U, w, VT);
    }
    static int InvertMatrix(double** a, double** ai, int n) { return rmath::lu_invert(a, ai, n); }
    static int JacobiN(double** a, int n, double* w, double** v) { return rmath::jacobi_upper(a, n, w, v); }
    static void Diagonalize3x3(const double[3][3], double[3], double[3][3]) {
        std::cerr << "shim vtkMath: Diagonalize3x3 (curvature by normal analysis) is not available" << std::endl;
        std::abort();
    }
    // Random numbers (only the non-default InitialSamplingType 0 uses them):
    // a 64-bit LCG, not VTK's generator.
    static void RandomSeed(int s) { state() = (unsigned long long)s; }
    static double Random() {
        state() = state() * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(state() >> 11) * (1.0 / 9007199254740992.0);
    }
    static double Random(double a, double b) { return a + (b - a) * Random(); }
private:
    static unsigned long long& state() { static unsigned long long s = 1; return s; }
};

class vtkTriangle {
public:
    static double TriangleArea(const double p1[3], const double p2[3], const double p3[3]) {
        return rmath::tri_area(p1, p2, p3);
    }
    static void ComputeQuadric(const double x1[3], const double x2[3], const double x3[3], double q[4][4]) {
        rmath::tri_quadric(x1, x2, x3, q);
    }
    static void ComputeNormal(const double x1[3], const double x2[3], const double x3[3], double n[3]) {
        rmath::tri_normal(x1, x2, x3, n);
    }
};

class vtkDataSetAttributes : public vtkObject {
public:
    void SetScalars(vtkDataArray*) {}
    void Initialize() {}
};
class vtkCellData : public vtkDataSetAttributes {};
class vtkPointData : public vtkDataSetAttributes {};

// Compile-only: the principal-direction display polydata of vtkCurvatureMeasure.
class vtkPoints : public vtkObject {
public:
    static vtkPoints* New() { return new vtkPoints; }
    void Allocate(vtkIdType) {}
    vtkIdType InsertNextPoint(const double p[3]) { P.insert(P.end(), p, p + 3); return (vtkIdType)P.size() / 3 - 1; }
    void ComputeBounds() {}
    double* GetBounds() { return B; }
    void GetBounds(double b[6]) { for (int i = 0; i < 6; i++) b[i] = B[i]; }
    double B[6] = {0, 0, 0, 0, 0, 0};
private:
    std::vector<double> P;
};

class vtkPolyData : public vtkObject {
public:
    static vtkPolyData* New() { return new vtkPolyData; }
    vtkCellData* GetCellData() { return &CD; }
    vtkPointData* GetPointData() { return &PD; }
    void ShallowCopy(vtkPolyData*) {}
    void Allocate(vtkIdType) {}
    void SetPoints(vtkPoints* p) { Pts = p; }
    vtkPoints* GetPoints() { return Pts; }
    vtkIdType InsertNextCell(int, vtkIdList*) { return 0; }
    vtkPoints* Pts = nullptr;
private:
    vtkCellData CD;
    vtkPointData PD;
};

class vtkTriangleFilter : public vtkObject {
public:
    static vtkTriangleFilter* New() { return new vtkTriangleFilter; }
    void SetInputData(vtkPolyData* p) { In = p; }
    void PassVertsOff() {}
    void Update() {}
    vtkPolyData* GetOutput() { return In; }
private:
    vtkPolyData* In = nullptr;
};

class vtkMultiThreader : public vtkObject {
public:
    struct ThreadInfo { int ThreadID; int NumberOfThreads; void* UserData; };
    typedef void* (*ThreadFunctionType)(void*);
    static vtkMultiThreader* New() { return new vtkMultiThreader; }
    static int GetGlobalDefaultNumberOfThreads() { return (int)std::max(1u, std::thread::hardware_concurrency()); }
    int GetNumberOfThreads() { return NumberOfThreads; }
    void SetNumberOfThreads(int n) { NumberOfThreads = n; }
    void SetSingleMethod(ThreadFunctionType f, void* data) { Fn = f; Data = data; }
    void SingleMethodExecute() {
        std::vector<std::thread> th;
        std::vector<ThreadInfo> info(NumberOfThreads);
        for (int i = 0; i < NumberOfThreads; i++) {
            info[i] = {i, NumberOfThreads, Data};
            th.emplace_back(Fn, (void*)&info[i]);
        }
        for (auto& t : th) t.join();
    }
private:
    int NumberOfThreads = GetGlobalDefaultNumberOfThreads();
    ThreadFunctionType Fn = nullptr;
    void* Data = nullptr;
};

// Max-priority queue of ids (the subset of vtkPriorityQueue the reference calls).
class vtkPriorityQueue : public vtkObject {
public:
    static vtkPriorityQueue* New() { return new vtkPriorityQueue; }
    void Allocate(vtkIdType n, vtkIdType = 1000) { H.reserve(n); }
    // an id already in the queue is not inserted again (the threaded engine re-inserts
    // every region at each FillQueuesFromClustering)
    void Insert(double priority, vtkIdType id) {
        for (const auto& h : H)
            if (h.second == id) return;
        H.push_back({priority, id});
        std::push_heap(H.begin(), H.end(), cmp);
    }
    vtkIdType Pop(vtkIdType = 0) {
        if (H.empty()) return -1;
        std::pop_heap(H.begin(), H.end(), cmp);
        const vtkIdType id = H.back().second;
        H.pop_back();
        return id;
    }
    vtkIdType Pop(vtkIdType, double& priority) {
        if (H.empty()) return -1;
        std::pop_heap(H.begin(), H.end(), cmp);
        priority = H.back().first;
        const vtkIdType id = H.back().second;
        H.pop_back();
        return id;
    }
    vtkIdType GetNumberOfItems() { return (vtkIdType)H.size(); }
    void Reset() { H.clear(); }
private:
    // vtkPriorityQueue pops the smallest priority first
    static bool cmp(const std::pair<double, vtkIdType>& a, const std::pair<double, vtkIdType>& b) { return a.first > b.first; }
    std::vector<std::pair<double, vtkIdType>> H;
};

class vtkLookupTable : public vtkObject {
public:
    static vtkLookupTable* New() { return new vtkLookupTable; }
    void SetTableRange(double, double) {}
    void SetSaturationRange(double, double) {}
    void SetHueRange(double, double) {}
    void SetValueRange(double, double) {}
    void SetScaleToLog10() {}
    void Build() {}
};
