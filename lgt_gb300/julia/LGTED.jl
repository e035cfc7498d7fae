# LGTED.jl -- Julia binding of liblgted.so (include/lgt_ed.h).
#
# Drop-in methods for the exact-diagonalisation entry points of finite_ed.jl:
# the same names and argument meaning, dispatching on handle types instead of
# Vector{NamedTuple} / SparseMatrixCSC.  Include it after (or instead of) the
# ED section of finite_ed.jl:
#
#     include("LGTED.jl"); using .LGTED
#     states, key_dict = LGTED.build_basis(3, 4, 1, g_charges)
#     H  = LGTED.build_hamiltonian(states, key_dict, 3, 4, 1; g=1.0, t=1.0, m=2.0)
#     E0, ψ0 = LGTED.find_ground_state(H)
#     data = LGTED.evolve_ED!(copy(ψ0), H, states, 3, 4, 1; dt=0.02, n_steps=2)
#
# Set ENV["LGTED_LIB"] to the path of liblgted.so (default: next to this file).
module LGTED

const libpath = get(ENV, "LGTED_LIB", joinpath(@__DIR__, "..", "liblgted.so"))

const LGT_OK = Int32(0)
const LGT_ERR_NOCONV = Int32(6)
const LGT_MODEL_REF = UInt32(0)
const LGT_MODEL_PJW = UInt32(3)
const LGT_FP64 = Int32(0)
const LGT_FP32_MIXED = Int32(2)

struct KrylovOpts
    krylovdim::Int32
    maxiter::Int32
    tol::Float64
    precision::Int32
    reorth_passes::Int32
    check_every::Int32
    refine_steps::Int32
    seed::UInt64
    use_graph::Int32
    start_given::Int32
    solver::Int32
end

struct Info
    matvecs::Int64
    restarts::Int32
    converged::Int32
    max_residual::Float64
    seconds::Float64
end

struct Obs
    t::Float64
    nf_mean::Float64
    nf_even::Float64
    nf_odd::Float64
    E2_mean::Float64
    plaq_mean::Float64
    n_stag::Float64
    norm2::Float64
end

last_error() = unsafe_string(ccall((:lgt_last_error, libpath), Cstring, ()))

function check(code::Int32)
    code == LGT_OK && return nothing
    # the reference's @assert failures become exceptions here as well
    code == LGT_ERR_NOCONV && throw(AssertionError("Ground-state eigsolve did not converge: " * last_error()))
    throw(ErrorException("lgted error $code: " * last_error()))
end

function defaults(for_exponentiate::Bool)
    r = Ref{KrylovOpts}()
    ccall((:lgt_krylov_defaults, libpath), Cvoid, (Ref{KrylovOpts}, Cint), r, for_exponentiate)
    return r[]
end

# ── basis: build_basis (finite_ed.jl:125-162) ───────────────────────────────
mutable struct Basis
    ptr::Ptr{Cvoid}
    nx::Int
    ny::Int
    dg::Int
    dim::Int
    function Basis(ptr, nx, ny, dg, dim)
        b = new(ptr, nx, ny, dg, dim)
        finalizer(b -> ccall((:lgt_basis_destroy, libpath), Cvoid, (Ptr{Cvoid},), b.ptr), b)
        return b
    end
end
Base.length(b::Basis) = b.dim

"Dict-like view of the reference key_dict: _encode key => 1-based index."
struct KeyDict <: AbstractDict{Int64,Int}
    basis::Basis
end
function lookup(kd::KeyDict, keys::Vector{Int64})
    out = zeros(Int64, length(keys))
    check(ccall((:lgt_basis_lookup, libpath), Int32, (Ptr{Cvoid}, Ptr{Int64}, Int64, Ptr{Int64}),
                kd.basis.ptr, keys, length(keys), out))
    return out
end
Base.haskey(kd::KeyDict, k::Int64) = lookup(kd, [k])[1] != 0
function Base.getindex(kd::KeyDict, k::Int64)
    i = lookup(kd, [k])[1]
    i == 0 && throw(KeyError(k))
    return Int(i)
end
Base.length(kd::KeyDict) = kd.basis.dim

function build_basis(nx::Int, ny::Int, dg::Int, g_charges::Matrix{Int})
    g = Int32.(g_charges)                       # column-major, as lgt_ed.h expects
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lgt_basis_create, libpath), Int32,
                (Int32, Int32, Int32, Ptr{Int32}, Int32, Ref{Ptr{Cvoid}}),
                nx, ny, dg, g, -1, out))
    dim = Ref{Int64}(0)
    check(ccall((:lgt_basis_dim, libpath), Int32, (Ptr{Cvoid}, Ref{Int64}), out[], dim))
    b = Basis(out[], nx, ny, dg, Int(dim[]))
    return b, KeyDict(b)
end

# ── Hamiltonian: build_hamiltonian (finite_ed.jl:252-322) ──────────────────
mutable struct Hamiltonian
    ptr::Ptr{Cvoid}
    basis::Basis
    K::Int
    function Hamiltonian(ptr, basis, K)
        h = new(ptr, basis, K)
        finalizer(h -> ccall((:lgt_ham_destroy, libpath), Cvoid, (Ptr{Cvoid},), h.ptr), h)
        return h
    end
end
Base.size(H::Hamiltonian) = (H.basis.dim, H.basis.dim)

function build_hamiltonian(states::Basis, key_dict::KeyDict, nx::Int, ny::Int, dg::Int;
                           g, t, m, model::UInt32=LGT_MODEL_REF)
    gs, ts, ms = Float64.(collect(g)), Float64.(collect(t)), Float64.(collect(m))
    K = max(length(gs), length(ts), length(ms))
    gs, ts, ms = (length(v) == 1 ? fill(v[1], K) : v for v in (gs, ts, ms))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lgt_ham_create, libpath), Int32,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, UInt32, Ref{Ptr{Cvoid}}),
                states.ptr, K, gs, ts, ms, model, out))
    return Hamiltonian(out[], states, K)
end

"nnz(H) as SparseArrays counts it (finite_ed.jl:355)."
function nnz(H::Hamiltonian)
    n = Ref{Int64}(0)
    check(ccall((:lgt_ham_nnz, libpath), Int32, (Ptr{Cvoid}, Ref{Int64}), H.ptr, n))
    return Int(n[])
end

"Autotuner report for H's Krylov panels (ncomp 1: ground states, 2: exp steps); tunes on first use."
struct Tuning
    hpsi_kernel::Int32
    reduce_blocks::Int32
    hpsi_ms::Float64
    reduce_ms::Float64
    measured::Int32
end

"Names of the `hpsi_kernel` codes of `Tuning` (index = code + 1; include/lgt_ed.h)."
const HPSI_KERNELS = ("rule", "generic", "fixed_vpl1", "fixed_vpl2", "fixed_wide",
                      "table_vpl1", "table_vpl2", "table_wide", "table_gather")

function autotune(H::Hamiltonian; ncomp::Integer=1, precision::Int32=LGT_FP64)
    t = Ref{Tuning}()
    check(ccall((:lgt_autotune, libpath), Int32, (Ptr{Cvoid}, Int32, Int32, Ref{Tuning}),
                H.ptr, Int32(ncomp), precision, t))
    return t[]
end

# ── find_ground_state (finite_ed.jl:333-341) ────────────────────────────────
function find_ground_state(H::Hamiltonian; tol=1e-10, krylovdim=50, maxiter=300,
                           precision::Int32=LGT_FP64, seed::Integer=0)
    o = defaults(false)
    o = KrylovOpts(krylovdim, maxiter, tol, precision, o.reorth_passes, o.check_every,
                   o.refine_steps, UInt64(seed), o.use_graph, 0, 0)
    N, K = H.basis.dim, H.K
    E0 = zeros(Float64, K)
    ψ = zeros(Float64, K, N)                      # [k, row]: row-major panel [N][K]
    info = Ref{Info}()
    check(ccall((:lgt_ground_state, libpath), Int32,
                (Ptr{Cvoid}, Ref{KrylovOpts}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, UInt32, Ref{Info}),
                H.ptr, Ref(o), E0, ψ, C_NULL, 0, info))
    vecs = [ComplexF64.(ψ[k, :]) for k in 1:K]
    return K == 1 ? (E0[1], vecs[1]) : (E0, vecs)
end

function ite_ground_state_ED(states, key_dict, nx, ny, dg; g, t, m)
    H = build_hamiltonian(states, key_dict, nx, ny, dg; g=g, t=t, m=m)
    return find_ground_state(H)
end

# ── find_ground_state then measure_ED of its state, as gs_benchmark.jl:116-125
#    runs them per point, in one call (lgt_ground_state_observe) ─────────────
function find_ground_state_measured(H::Hamiltonian; tol=1e-10, krylovdim=50, maxiter=300,
                                    precision::Int32=LGT_FP64, seed::Integer=0)
    o = defaults(false)
    o = KrylovOpts(krylovdim, maxiter, tol, precision, o.reorth_passes, o.check_every,
                   o.refine_steps, UInt64(seed), o.use_graph, 0, 0)
    N, K = H.basis.dim, H.K
    nx, ny = H.basis.nx, H.basis.ny
    E0 = zeros(Float64, K)
    ψ = zeros(Float64, K, N)                      # [k, row]: row-major panel [N][K]
    nf = zeros(Float64, nx * ny, K)
    e2 = zeros(Float64, nx * ny, K)
    obs = Vector{Obs}(undef, K)
    info = Ref{Info}()
    check(ccall((:lgt_ground_state_observe, libpath), Int32,
                (Ptr{Cvoid}, Ref{KrylovOpts}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, UInt32,
                 Ref{Info}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Obs}),
                H.ptr, Ref(o), E0, ψ, C_NULL, 0, info, nf, e2, C_NULL, obs))
    vecs = [ComplexF64.(ψ[k, :]) for k in 1:K]
    recs = [(t=0.0, nf_mean=obs[k].nf_mean, nf_even=obs[k].nf_even, nf_odd=obs[k].nf_odd,
             E2_mean=obs[k].E2_mean, nf_grid=reshape(nf[:, k], nx, ny),
             E2_grid=reshape(e2[:, k], nx, ny)) for k in 1:K]
    return K == 1 ? (E0[1], vecs[1], recs[1]) : (E0, vecs, recs)
end

# ── measure_ED (finite_ed.jl:369-393) ───────────────────────────────────────
function measure_ED(ψ::Vector{ComplexF64}, states::Basis, nx::Int, ny::Int, dg::Int,
                    t_now::Float64; H::Union{Nothing,Hamiltonian}=nothing)
    Hobs = H === nothing ? build_hamiltonian(states, KeyDict(states), nx, ny, dg; g=1.0, t=1.0, m=1.0) : H
    nf = zeros(Float64, nx * ny)
    e2 = zeros(Float64, nx * ny)
    s = Ref{Obs}()
    check(ccall((:lgt_observe, libpath), Int32,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Int32, Int32, UInt32, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Obs}),
                Hobs.ptr, ψ, 2, LGT_FP64, 0, t_now, nf, e2, C_NULL, s))
    o = s[]
    return (t=t_now, nf_mean=o.nf_mean, nf_even=o.nf_even, nf_odd=o.nf_odd, E2_mean=o.E2_mean,
            nf_grid=reshape(nf, nx, ny), E2_grid=reshape(e2, nx, ny))
end

# ── evolve_ED! (finite_ed.jl:405-431) ───────────────────────────────────────
function evolve_ED!(ψ::Vector{ComplexF64}, H::Hamiltonian, states::Basis, nx::Int, ny::Int,
                    dg::Int; dt::Float64, n_steps::Int, measure_every::Int=10)
    o = defaults(true)
    R = (n_steps + 1) * H.K
    obs = Vector{Obs}(undef, R)
    nf = zeros(Float64, nx * ny, R)
    e2 = zeros(Float64, nx * ny, R)
    info = Ref{Info}()
    ψw = copy(ψ)   # the reference rebinds ψ inside evolve_ED!, leaving the caller's vector as is
    check(ccall((:lgt_expm_steps_grids, libpath), Int32,
                (Ptr{Cvoid}, Ref{KrylovOpts}, Float64, Int32, Ptr{ComplexF64}, Ptr{Obs},
                 Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, UInt32, Ref{Info}),
                H.ptr, Ref(o), dt, n_steps, ψw, obs, nf, e2, C_NULL, C_NULL, 0, info))
    return [(t=obs[i].t, nf_mean=obs[i].nf_mean, nf_even=obs[i].nf_even, nf_odd=obs[i].nf_odd,
             E2_mean=obs[i].E2_mean, nf_grid=reshape(nf[:, i], nx, ny),
             E2_grid=reshape(e2[:, i], nx, ny))
            for i in 1:R]
end

end # module
