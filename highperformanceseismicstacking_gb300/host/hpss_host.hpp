// hpss_host.hpp -- C++ host side of the GB300 engine, mirroring the
// reference's host interfaces for the semblance path so that its CLI, SU
// input/output and compute-algorithm flow are a drop-in:
//
//   model      Trace / Cdp / Gather       (common/include/model/*.hpp)
//   traveltime Traveltime + CMP / ZO-CRS / OCT / stretch-free wrapper,
//              TraveltimeBuilder          (common/include/traveltime/*.hpp)
//   algorithm  DeviceContext, ComputeAlgorithm, LinearSearchAlgorithm,
//              DifferentialEvolutionAlgorithm, StretchFreeAlgorithm,
//              ComputeAlgorithmBuilder    (common/include/semblance/**)
//   output     Logger, StatisticResult, MidpointResult, ResultSet, Dumper
//   cli        Parser (+ LinearSearch / DifferentialEvolution / StretchFree),
//              SingleHostRunner           (common/include/parser, execution)
//
// The compute algorithms call the engine only through the C ABI in
// include/hpss.h.  Beyond the reference's per-midpoint entry
// (computeSemblanceAndParametersForMidpoint) they offer a batched entry that
// computes all midpoints of a device in one call.
#pragma once

#include <chrono>
#include <sstream>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/hpss.h"

namespace hpsshost {

// ----------------------------------------------------------------- logging
enum class LogLevel { ERROR, INFO, LOW, HIGH, DEBUG };

class Logger {
  public:
    static Logger *getInstance();
    LogLevel getVerbosity() const { return verbosity; }
    void setVerbosity(LogLevel v) { verbosity = v; }
    static void print(LogLevel lvl, const std::string &message);

  private:
    LogLevel verbosity = LogLevel::INFO;
};

#define HPSS_LOG(level, message)                                              \
    do {                                                                      \
        if ((level) <= ::hpsshost::Logger::getInstance()->getVerbosity()) {   \
            std::ostringstream _s;                                            \
            _s << message;                                                    \
            ::hpsshost::Logger::print(level, _s.str());                       \
        }                                                                     \
    } while (0)
#define LOGE(m) HPSS_LOG(::hpsshost::LogLevel::ERROR, m)
#define LOGI(m) HPSS_LOG(::hpsshost::LogLevel::INFO, m)
#define LOGL(m) HPSS_LOG(::hpsshost::LogLevel::LOW, m)
#define LOGH(m) HPSS_LOG(::hpsshost::LogLevel::HIGH, m)
#define LOGD(m) HPSS_LOG(::hpsshost::LogLevel::DEBUG, m)

// ----------------------------------------------------------------- model
// SU trace header: the 240-byte trace_info_t of the reference
// (common/include/model/Trace.hpp:9-91), a file format.
#pragma pack(push, 1)
struct trace_info_t {
    int32_t tracl, tracr, fldr, tracf, ep, cdp, cdpt;
    int16_t trid, nvs, nhs, duse;
    int32_t offset, gelev, selev, sdepth, gdel, sdel, swdep, gwdep;
    int16_t scalel, scalco;
    int32_t sx, sy, gx, gy;
    int16_t counit, wevel, swevel, sut, gut, sstat, gstat, tstat, laga, lagb, delrt, muts,
        mute;
    uint16_t ns, dt;
    int16_t gain, igc, igi, corr, sfs, sfe, slen, styp, stas, stae, tatyp, afilf, afils,
        nofilf, nofils, lcf, hcf, lcs, hcs, year, day, hour, minute, sec, timbas, trwf, grnors,
        grnofr, grnlof, gaps, otrav;
    float d1, f1, d2, f2, ungpow, unscale;
    int32_t ntr;
    int16_t mark, shortpad;
    int16_t unass[14];
};
#pragma pack(pop)
static_assert(sizeof(trace_info_t) == 240, "SU header is 240 bytes");

namespace Utils {
float midpoint(const trace_info_t &info, float azimuthInRad);
float halfoffset(const trace_info_t &info, float azimuthInRad);
float degreesToRad(float degree);
}  // namespace Utils

class Trace {
  public:
    Trace();
    bool read(std::ifstream &fin, float azimuthInRad);  // false at end of file
    float getMidpoint() const { return midpoint; }
    float getHalfoffset() const { return halfoffset; }
    const trace_info_t &getInfo() const { return info; }
    const std::vector<float> &getSamples() const { return samples; }
    unsigned int getSampleCount() const { return (unsigned)samples.size(); }
    bool isMidpointInRange(float lower, float upper) const {
        return midpoint >= lower && midpoint <= upper;
    }
    bool operator<(const Trace &o) const;

  private:
    float halfoffset = 0, midpoint = 0;
    std::vector<float> samples;
    trace_info_t info;
};

class Cdp {
  public:
    Cdp() = default;
    Cdp(float m, const trace_info_t &i) : midpoint(m), cdpInfo(i) {}
    const trace_info_t &getCdpInfo() const { return cdpInfo; }
    void incrementTraceCountBy(unsigned s) { traceCount += s; }
    void incrementSampleCountBy(unsigned s) { sampleCount += s; }
    unsigned getTraceCount() const { return traceCount; }

  private:
    float midpoint = 0;
    trace_info_t cdpInfo{};
    unsigned sampleCount = 0, traceCount = 0;
};

// Gather::readGatherFromFile semantics (common/src/model/Gather.cpp:49-126).
class Gather {
  public:
    static Gather *getInstance();
    void readGatherFromFile(const std::string &file);
    void setApm(float v) { apm = v; }
    void setAph(float v) { aph = v; }
    void setTau(float v) { tau = v; }
    void setAzimuthInDegree(float deg);
    void setLowestAllowedMidpoint(float v) { lowestAllowedMidpoint = v; }
    void setBiggestAllowedMidpoint(float v) { biggestAllowedMidpoint = v; }
    float getApm() const { return apm; }
    float getAzimuthInRad() const { return azimuthInRad; }
    int getTauIndexDisplacement() const { return tauIndexDisplacement; }
    unsigned getWindowSize() const { return (unsigned)windowSize; }
    unsigned getSamplesPerTrace() const { return samplesPerTrace; }
    float getSamplePeriodInSeconds() const { return dtInSeconds; }
    unsigned getTotalTracesCount() const { return (unsigned)traces.size(); }
    const std::map<float, Cdp> &getCdps() const { return cdps; }
    const Trace &getTraceAtIndex(unsigned i) const { return traces[i]; }
    const std::string toString() const;
    void reset();

  private:
    float apm = 0, aph = 0, azimuthInDegrees = 0, azimuthInRad = 0;
    unsigned short dt = 0;
    float dtInSeconds = 0;
    float lowestAllowedMidpoint, biggestAllowedMidpoint;
    unsigned samplesCount = 0, samplesPerTrace = 0;
    float tau = 0;
    int tauIndexDisplacement = 0, windowSize = 1;
    std::map<float, Cdp> cdps;
    std::vector<Trace> traces;

  public:
    Gather();
};

// ----------------------------------------------------------------- traveltime
enum traveltime_t { CMP = 0, ZOCRS = 1, OCT = 2 };

class TraveltimeParameter {
  public:
    explicit TraveltimeParameter(const std::string &d) : description(d) {}
    void updateMinimum(float v) { minimum = v; }
    void updateMaximum(float v) { maximum = v; }
    float getMinimum() const { return minimum; }
    float getMaximum() const { return maximum; }
    const std::string &getParameterDescription() const { return description; }

  private:
    float minimum = 0, maximum = 0;
    std::string description;
};

class Traveltime {
  public:
    virtual ~Traveltime() = default;
    virtual unsigned getNumberOfParameters() const { return (unsigned)params.size(); }
    unsigned getNumberOfCommonResults() const { return 2; }
    virtual unsigned getNumberOfResults() const { return 2 + getNumberOfParameters(); }
    virtual std::string getDescriptionForResult(unsigned i) const;
    std::string getDescriptionForParameter(unsigned i) const {
        return params[i].getParameterDescription();
    }
    virtual float getReferenceHalfoffset() const { return referenceHalfOffset; }
    void updateLowerBoundForParameter(unsigned p, float v) { params[p].updateMinimum(v); }
    void updateUpperBoundForParameter(unsigned p, float v) { params[p].updateMaximum(v); }
    virtual float getLowerBoundForParameter(unsigned p) const { return params[p].getMinimum(); }
    virtual float getUpperBoundForParameter(unsigned p) const { return params[p].getMaximum(); }
    virtual std::string getTraveltimeWord() const = 0;
    virtual void updateReferenceHalfoffset(float h0) = 0;
    virtual traveltime_t getModel() const = 0;
    virtual std::string toString() const;

  protected:
    explicit Traveltime(std::vector<TraveltimeParameter> v) : params(std::move(v)) {}
    std::vector<TraveltimeParameter> params;
    float referenceHalfOffset = 0;
};

class CommonMidPoint : public Traveltime {
  public:
    static constexpr unsigned VELOCITY = 0;
    CommonMidPoint() : Traveltime({TraveltimeParameter("velocity")}) {}
    std::string getTraveltimeWord() const override { return "cmp"; }
    void updateReferenceHalfoffset(float) override {}
    traveltime_t getModel() const override { return CMP; }
};

class CommonReflectionSurface : public Traveltime {
  public:
    static constexpr unsigned VELOCITY = 0, A = 1, B = 2;
    CommonReflectionSurface()
        : Traveltime({TraveltimeParameter("velocity"), TraveltimeParameter("a"),
                      TraveltimeParameter("b")}) {}
    std::string getTraveltimeWord() const override { return "zocrs"; }
    void updateReferenceHalfoffset(float) override {}
    traveltime_t getModel() const override { return ZOCRS; }
    float v0 = 0, ainDeg = 0, bpctg = 0;
    std::string toString() const override;
};

class OffsetContinuationTrajectory : public Traveltime {
  public:
    static constexpr unsigned VELOCITY = 0, SLOPE = 1;
    OffsetContinuationTrajectory()
        : Traveltime({TraveltimeParameter("velocity"), TraveltimeParameter("slope")}) {}
    std::string getTraveltimeWord() const override { return "oct"; }
    void updateReferenceHalfoffset(float h0) override { referenceHalfOffset = h0; }
    traveltime_t getModel() const override { return OCT; }
};

// Stretch-free wrapper: results are (coherence, stack, n) -- three rows.  (The
// reference sizes them 2 + nParams, an out-of-bounds read for ZO-CRS/OCT;
// StretchFreeAlgorithm.cpp:60 vs SingleHostRunner.cpp:137.)
class StretchFreeTraveltimeWrapper : public Traveltime {
  public:
    explicit StretchFreeTraveltimeWrapper(Traveltime *t)
        : Traveltime({TraveltimeParameter("n")}), wrapped(t) {}
    unsigned getNumberOfParameters() const override { return wrapped->getNumberOfParameters(); }
    unsigned getNumberOfResults() const override { return 3; }
    std::string getDescriptionForResult(unsigned i) const override;
    float getReferenceHalfoffset() const override { return wrapped->getReferenceHalfoffset(); }
    float getLowerBoundForParameter(unsigned p) const override {
        return wrapped->getLowerBoundForParameter(p);
    }
    float getUpperBoundForParameter(unsigned p) const override {
        return wrapped->getUpperBoundForParameter(p);
    }
    std::string getTraveltimeWord() const override {
        return "stretch_free_" + wrapped->getTraveltimeWord();
    }
    void updateReferenceHalfoffset(float h0) override { wrapped->updateReferenceHalfoffset(h0); }
    traveltime_t getModel() const override { return wrapped->getModel(); }
    std::string toString() const override { return wrapped->toString(); }

  private:
    std::unique_ptr<Traveltime> wrapped;
};

// TraveltimeBuilder (common/src/traveltime/TraveltimeBuilder.cpp:24-106).
namespace TraveltimeBuilder {
Traveltime *buildCommonMidPoint(const std::vector<float> &lo, const std::vector<float> &hi);
Traveltime *buildZeroOffsetCommonReflectionSurface(const std::vector<float> &lo,
                                                   const std::vector<float> &hi, float v0,
                                                   float aIn, float bPctg);
Traveltime *buildOffsetContinuationTrajectory(const std::vector<float> &lo,
                                              const std::vector<float> &hi, float h0);
}  // namespace TraveltimeBuilder

// ----------------------------------------------------------------- results
enum class StatisticResult {
    EFFICIENCY,
    INTR_PER_SEC,
    SELECTED_TRACES,
    TOTAL_SELECTION_KERNEL_EXECUTION_TIME,
    TOTAL_KERNEL_EXECUTION_TIME,
    CNT
};
const std::string &statisticName(StatisticResult r);

class MidpointResult {
  public:
    void save(float m0, std::vector<float>::const_iterator b, std::vector<float>::const_iterator e) {
        results[m0].assign(b, e);
    }
    const std::vector<float> &get(float m0) const;

  private:
    std::map<float, std::vector<float>> results;
};

class StatisticalMidpointResult {
  public:
    void setStatisticalResultForMidpoint(float m0, float v) { stats[m0] = v; }
    float getStatisticalResultForMidpoint(float m0) const;
    float getAverageOfAllMidpoints() const;

  private:
    std::map<float, float> stats;
};

class ResultSet {
  public:
    ResultSet(unsigned numberOfResults, unsigned samples)
        : resultArray(numberOfResults), samplesPerResult(samples) {}
    void setAllResultsForMidpoint(float m0, const std::vector<float> &array, size_t offset = 0);
    void setStatisticalResultForMidpoint(float m0, StatisticResult s, float v) {
        stats[s].setStatisticalResultForMidpoint(m0, v);
    }
    const MidpointResult &getArrayForResult(unsigned i) const { return resultArray[i]; }
    const StatisticalMidpointResult &get(StatisticResult s) const;

  private:
    std::vector<MidpointResult> resultArray;
    std::map<StatisticResult, StatisticalMidpointResult> stats;
    unsigned samplesPerResult;
};

// ----------------------------------------------------------------- devices + algorithms
// A device context owns the engine handle of its device (the reference's
// CudaDeviceContext::activate selects the device, CudaDeviceContext.cu:14-17).
class DeviceContext {
  public:
    explicit DeviceContext(unsigned devId);
    ~DeviceContext();
    void activate() const {}
    hpss_handle handle() const { return h; }
    unsigned getDeviceId() const { return deviceId; }

  private:
    unsigned deviceId;
    hpss_handle h = nullptr;
};

void check(hpss_handle h, hpss_status rc);  // status -> the reference's exceptions

class ComputeAlgorithm {
  public:
    ComputeAlgorithm(const std::string &name, std::shared_ptr<Traveltime> model,
                     std::shared_ptr<DeviceContext> ctx, unsigned threadCount);
    virtual ~ComputeAlgorithm() = default;
    bool isSetUp() const { return isSet; }
    const std::string &getAlgorithmName() const { return algorithmName; }
    const std::vector<float> &getComputedResults() const { return computedResults; }
    float getStatisticalResult(StatisticResult r) const;
    virtual void compileKernels(const std::string &) {}
    virtual void setUp();
    virtual void computeSemblanceAndParametersForMidpoint(float m0);
    // the selection and evaluation run inside the batched engine call
    virtual void computeSemblanceAtGpuForMidpoint(float) {}
    virtual void selectTracesToBeUsedForMidpoint(float) {}
    // All midpoints in one engine call; results [n][rows][S], per-midpoint stats.
    virtual void computeSemblanceAndParametersForMidpoints(const std::vector<float> &m0s,
                                                           std::vector<float> &results,
                                                           std::vector<std::map<StatisticResult, float>> &stats) = 0;
    virtual std::string toString() const = 0;
    unsigned resultRows() const { return traveltime->getNumberOfResults(); }
    // engine options (no reference counterpart): amplitude storage
    // (HPSS_STORAGE_*) and linear-search grid (HPSS_GRID_*), applied by setUp
    void setEngineStorage(int s) { storage = s; }
    void setEngineGridMode(int m) { gridMode = m; }
    void setEnginePrecision(int flags) { precisionFlags = flags; }

  protected:
    void fillStats(const std::vector<float> &m0s, const hpss_stats &st, double perCandidateFactor,
                   std::vector<std::map<StatisticResult, float>> &stats);
    bool isSet = false;
    std::string algorithmName;
    std::shared_ptr<DeviceContext> deviceContext;
    std::shared_ptr<Traveltime> traveltime;
    unsigned threadCount;
    std::vector<float> computedResults;
    std::unordered_map<int, float> computedStatisticalResults;
    int storage = HPSS_STORAGE_FP32;
    int gridMode = HPSS_GRID_REFERENCE;
    int precisionFlags = 0;
};

class LinearSearchAlgorithm : public ComputeAlgorithm {
  public:
    LinearSearchAlgorithm(std::shared_ptr<Traveltime> model, std::shared_ptr<DeviceContext> ctx,
                          unsigned threadCount, const std::vector<int> &granularity,
                          int kernel = HPSS_KERNEL_TUNED);
    void computeSemblanceAndParametersForMidpoints(
        const std::vector<float> &m0s, std::vector<float> &results,
        std::vector<std::map<StatisticResult, float>> &stats) override;
    unsigned getTotalNumberOfParameters() const;
    std::string toString() const override;

  private:
    std::vector<uint32_t> granularity;
    int kernel;
};

class DifferentialEvolutionAlgorithm : public ComputeAlgorithm {
  public:
    DifferentialEvolutionAlgorithm(std::shared_ptr<Traveltime> model,
                                   std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
                                   unsigned generations, unsigned population, float F, float CR,
                                   uint64_t seed);
    void computeSemblanceAndParametersForMidpoints(
        const std::vector<float> &m0s, std::vector<float> &results,
        std::vector<std::map<StatisticResult, float>> &stats) override;
    std::string toString() const override;

  private:
    unsigned generations, individualsPerPopulation;
    float F, CR;
    uint64_t seed;
};

class StretchFreeAlgorithm : public ComputeAlgorithm {
  public:
    StretchFreeAlgorithm(std::shared_ptr<Traveltime> model, std::shared_ptr<DeviceContext> ctx,
                         unsigned threadCount, const std::vector<std::string> &files);
    void setUp() override;
    void computeSemblanceAndParametersForMidpoints(
        const std::vector<float> &m0s, std::vector<float> &results,
        std::vector<std::map<StatisticResult, float>> &stats) override;
    std::string toString() const override;
    static constexpr int NMAX = 10;

  private:
    std::vector<std::string> parameterFileArray;
    std::map<float, std::vector<float>> nonStretchFreeParameters;  // [np][S] per midpoint
};

class ComputeAlgorithmBuilder {
  public:
    virtual ~ComputeAlgorithmBuilder() = default;
    virtual LinearSearchAlgorithm *buildLinearSearchAlgorithm(
        std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
        const std::vector<int> &discretization) = 0;
    virtual DifferentialEvolutionAlgorithm *buildDifferentialEvolutionAlgorithm(
        std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
        unsigned generations, unsigned population) = 0;
    virtual StretchFreeAlgorithm *buildStretchFreeAlgorithm(
        std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
        const std::vector<std::string> &files) = 0;
};

// Options beyond the reference's flags: --kernel, --seed, --de-f, --de-cr.
struct EngineOptions {
    int kernel = HPSS_KERNEL_TUNED;
    int storage = HPSS_STORAGE_FP32;
    int gridMode = HPSS_GRID_REFERENCE;
    int precisionFlags = 0;
    uint64_t seed = 0;
    bool seedGiven = false;
    float deF = 0.85f, deCR = 0.5f;
};

class Gb300ComputeAlgorithmBuilder : public ComputeAlgorithmBuilder {
  public:
    explicit Gb300ComputeAlgorithmBuilder(EngineOptions o = {}) : opts(o) {}
    LinearSearchAlgorithm *buildLinearSearchAlgorithm(std::shared_ptr<Traveltime>,
                                                      std::shared_ptr<DeviceContext>, unsigned,
                                                      const std::vector<int> &) override;
    DifferentialEvolutionAlgorithm *buildDifferentialEvolutionAlgorithm(
        std::shared_ptr<Traveltime>, std::shared_ptr<DeviceContext>, unsigned, unsigned,
        unsigned) override;
    StretchFreeAlgorithm *buildStretchFreeAlgorithm(std::shared_ptr<Traveltime>,
                                                    std::shared_ptr<DeviceContext>, unsigned,
                                                    const std::vector<std::string> &) override;
    EngineOptions opts;
};

// ----------------------------------------------------------------- output
class Dumper {
  public:
    Dumper(const std::string &path, const std::string &dataFile, const std::string &method,
           const std::string &traveltime);
    void createDir() const;
    void dumpGatherParameters(const std::string &file) const;
    void dumpTraveltime(const Traveltime *t) const;
    void dumpAlgorithm(const ComputeAlgorithm *a) const;
    void dumpResult(const std::string &name, const MidpointResult &r) const;
    void dumpStatisticalResult(const std::string &name, const StatisticalMidpointResult &r) const;
    const std::string &getOutputDirectoryPath() const { return outputDirectoryPath; }

  private:
    std::string outputDirectoryPath;
};

// ----------------------------------------------------------------- cli
class Parser {
  public:
    Parser();
    virtual ~Parser() = default;
    void parseArguments(int argc, const char *argv[]);
    std::string getFilename() const;
    std::string getInputFilePath() const;
    std::string getOutputDirectory() const;
    unsigned getGpuThreadCount() const;
    virtual Traveltime *parseTraveltime() const;
    void printHelp() const;
    void readGather() const;
    virtual ComputeAlgorithm *parseComputeAlgorithm(ComputeAlgorithmBuilder *builder,
                                                    std::shared_ptr<DeviceContext> ctx,
                                                    std::shared_ptr<Traveltime> tt) const = 0;
    virtual std::string getParserType() const = 0;
    EngineOptions engineOptions() const;

  protected:
    struct Option {
        std::string name, help;
        bool multi = false, required = false, flag = false;
        std::string def;
    };
    void add(const std::string &name, const std::string &help, bool required = false,
             bool multi = false, const std::string &def = "", bool flag = false);
    bool has(const std::string &n) const { return values.count(n) > 0; }
    std::string str(const std::string &n) const;
    float f(const std::string &n) const;
    unsigned u(const std::string &n) const;
    std::vector<float> floats(const std::string &n) const;
    std::vector<int> ints(const std::string &n) const;
    std::vector<Option> options;
    std::map<std::string, std::vector<std::string>> values;
};

class LinearSearchParser : public Parser {
  public:
    LinearSearchParser();
    ComputeAlgorithm *parseComputeAlgorithm(ComputeAlgorithmBuilder *, std::shared_ptr<DeviceContext>,
                                            std::shared_ptr<Traveltime>) const override;
    std::string getParserType() const override { return "greedy"; }
};

class DifferentialEvolutionParser : public Parser {
  public:
    DifferentialEvolutionParser();
    ComputeAlgorithm *parseComputeAlgorithm(ComputeAlgorithmBuilder *, std::shared_ptr<DeviceContext>,
                                            std::shared_ptr<Traveltime>) const override;
    std::string getParserType() const override { return "de"; }
};

class StretchFreeParser : public Parser {
  public:
    StretchFreeParser();
    Traveltime *parseTraveltime() const override;
    ComputeAlgorithm *parseComputeAlgorithm(ComputeAlgorithmBuilder *, std::shared_ptr<DeviceContext>,
                                            std::shared_ptr<Traveltime>) const override;
    std::string getParserType() const override { return "stretch_free"; }
};

// One worker thread per device; each takes a contiguous shard of the CDP
// midpoints and computes it in one engine call (the reference pops one
// midpoint at a time from a shared queue, SingleHostRunner.cpp:49-106).
class SingleHostRunner {
  public:
    explicit SingleHostRunner(Parser *p);
    int main(int argc, const char *argv[]);

  private:
    Parser *parser;
    std::shared_ptr<Traveltime> traveltime;
    std::unique_ptr<ResultSet> resultSet;
    std::mutex resultSetMutex;
};

}  // namespace hpsshost
