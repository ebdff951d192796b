#pragma once
// Rosenbrock tableaus of the perturbation kernel, in the transformed form of Hairer & Wanner
// (Solving ODEs II, IV.7, eq. 7.25) with W = 1/(hγ) I - J:
//   W U_i = f(t + c_i h, y + Σ_j A_ij U_j) + Σ_j (C_ij / h) U_j + h d_i ∂f/∂τ,
//   y1 = y + Σ_j m_j U_j,  error estimate = U_S (the embedded solution omits the last stage).
// Step-size control: fac = 0.9 err^-beta1 errold^beta2 on acceptance, max(0.2, 0.9 err^-rej) on
// rejection.  Accessors are constexpr: unrolled stage loops see the coefficients as immediates (zero
// entries fold away); rolled ones read a constant-memory copy built from the same accessors.
//
// Rodas5P (Steinebach 2023, order 5(4), stiffly accurate) is the reference's default integrator
// (src/solve.jl:320,339; OrdinaryDiffEqRosenbrock).  Its dense output here is an order-4
// continuous extension derived for this tableau (see dense()).
namespace sbz {
namespace ros {

struct Rodas5P {
  static constexpr int S = 8;
  static constexpr int NTIME = 5;  // distinct stage times after t: c2, c3, c4, c5 and t + h
  static constexpr int NDENSE = 3;
  static constexpr double gam = 0.21193756319429014;
  static constexpr double beta1 = 0.14, beta2 = 0.08, rej = 0.14;  // 7/(10·5), 2/(5·5)
  __host__ __device__ static constexpr double c(int i) {
    constexpr double v[8] = {0, 0.6358126895828704, 0.4095798393397535, 0.9769306725060716, 0.4288403609558664, 1, 1, 1};
    return v[i];
  }
  __host__ __device__ static constexpr double d(int i) {
    constexpr double v[8] = {0.21193756319429014, -0.42387512638858027, -0.3384627126235924, 1.8046452872882734,
                             2.325825639765069, 0, 0, 0};
    return v[i];
  }
  // stage time of stage i: 0 = t (the Jacobian set), q >= 1 = the q-th later time
  __host__ __device__ static constexpr int tslot(int i) {
    constexpr int v[8] = {0, 1, 2, 3, 4, 5, 5, 5};
    return v[i];
  }
  __host__ __device__ static constexpr double A(int i, int j) {
    constexpr double v[8][7] = {
        {0},
        {3.0},
        {2.849394379747939, 0.45842242204463923},
        {-6.954028509809101, 2.489845061869568, -10.358996098473584},
        {2.8029986275628964, 0.5072464736228206, -0.3988312541770524, -0.04721187230404641},
        {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946},
        {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0},
        {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0, 1.0}};
    return j < 7 ? v[i][j] : 0.0;
  }
  __host__ __device__ static constexpr double C(int i, int j) {
    constexpr double v[8][7] = {
        {0},
        {-14.155112264123755},
        {-17.97296035885952, -2.859693295451294},
        {147.12150275711716, -1.41221402718213, 71.68940251302358},
        {165.43517024871676, -0.4592823456491126, 42.90938336958603, -5.961986721573306},
        {24.854864614690072, -3.0009227002832186, 47.4931110020768, 5.5814197821558125, -0.6610691825249471},
        {30.91273214028599, -3.1208243349937974, 77.79954646070892, 34.28646028294783, -19.097331116725623,
         -28.087943162872662},
        {37.80277123390563, -3.2571969029072276, 112.26918849496327, 66.9347231244047, -40.06618937091002,
         -54.66780262877968, -9.48861652309627}};
    return j < 7 ? v[i][j] : 0.0;
  }
  // stage i's input is stage i-1's input plus U_{i-1} (stages 7 and 8)
  __host__ __device__ static constexpr bool incremental(int i) { return i >= 6; }
  // Order-4 continuous extension y(t + θh) = (1-θ) y + θ (y1 + (1-θ)(K0 + θ K1 + θ² K2)),
  // K_r = Σ_j H_rj U_j: the eight tree conditions of order <= 4 with θ-dependent weights
  // (Σ_j b_j(θ) Φ_j = P_t(θ), e.g. θ²/2 - γθ for the second-order tree) are linear in H for this
  // form and have rank 6 in the seven non-error stages; H u∞ = 0 (u∞: the stages of y' = λy as
  // hλ → -∞) completes them, so stiff components interpolate linearly between the step ends
  // instead of being amplified (the photon-baryon tight coupling).
  __host__ __device__ static constexpr double dense(int r, int j) {
    constexpr double v[3][8] = {
        {16.487964434865184, -2.370717139483559, -36.89699909384169, -47.19777482102162, 29.31762179544809, 37.62133721923128, 6.977388062974808, 0},
        {21.885022549967175, -1.5984168138259751, 162.13711388885017, 126.19157982265247, -76.60482233539331, -106.69765784722038, -28.805926606943324, 0},
        {-15.646484681406143, 3.423681775524067, -62.48695397162234, -48.12822622663184, 30.299848310633063, 44.62468119063477, 18.5833010918263, 0}};
    return v[r][j];
  }
};

}  // namespace ros
}  // namespace sbz
