# AmaruGPU.jl -- Julia binding of libamaru_gpu.so (include/amaru_gpu.h) for Amaru.jl.
#
# Loaded after `using Amaru`, it offers a GPU stage solver with the signature of
# mech_stage_solver! (src/mech/mech-solver.jl:186) and GPU versions of the three
# solver-level plugin functions the hot path calls:
#   mount_K(elems, ndofs)          src/mech/mech-solver.jl:78
#   update_state!(elems, dU, t)    src/mech/mech-solver.jl:124
#   solve_system!(K, U, F, nu)     src/solver.jl:5
# The element/material/stage API (FEModel, MechSolid, LinearElastic / VonMises /
# DruckerPrager, addstage!, solve!) is unchanged.  Elements or materials the
# library does not support raise an error: there is no CPU fallback.  Beside the
# static stage it runs the dynamic stage (dyn_stage_solver!), the modal solver
# (mech_modal_solver!), the nodal output recovery (nodal_patch_recovery) and the
# ascii VTU writer (save_vtu) on the library.
#
# Index convention: the C ABI is 0-based; this file converts (eq_id - 1).
module AmaruGPU

using Amaru
using DelimitedFiles
using SparseArrays

const LIB = get(ENV, "AMARU_GPU_LIB", joinpath(@__DIR__, "..", "amaru_gpu", "libamaru_gpu.so"))

const SHAPES = Dict("LIN2" => 1, "LIN3" => 2, "TRI3" => 3, "TRI6" => 4, "QUAD4" => 5, "QUAD8" => 6,
                    "QUAD9" => 7, "TET4" => 8, "TET10" => 9, "HEX8" => 10, "HEX20" => 11)
const STRESSMODELS = Dict(:d3 => 0, :planestrain => 1, :planestress => 2, :axisymmetric => 3)

struct ModelDesc
    ndim::Int32
    stressmodel::Int32
    thickness::Float64
    nnodes::Int64
    coords::Ptr{Float64}
    nelems::Int64
    shape::Ptr{Int32}
    nips::Ptr{Int32}
    conn_ptr::Ptr{Int64}
    conn::Ptr{Int64}
    mat_type::Ptr{Int32}
    mat_params::Ptr{Float64}
end

struct SolveOpts
    method::Int32
    rtol::Float64
    max_iters::Int32
    refine_every::Int32
end

struct SolveStats
    iterations::Int32
    refinements::Int32
    rel_residual::Float64
    seconds::Float64
end

struct StageParams
    tol::Float64; rtol::Float64; rspan::Float64; dT0::Float64; dTmin::Float64; dTmax::Float64
    scheme::Int32; maxits::Int32; autoinc::Int32; nincs::Int32; nouts::Int32
    linear::SolveOpts
end

mutable struct StageStats
    status::Int32; increments::Int32; iterations::Int32; krylov_iterations::Int32
    residue::Float64; T::Float64; seconds::Float64; solve_seconds::Float64
    StageStats() = new(0, 0, 0, 0, 0.0, 0.0, 0.0, 0.0)
end

mutable struct GPUModel
    h::Ptr{Cvoid}
    ndofs::Int
    nu::Int
    elems::Vector{Any}   # the elements on the device, in model order (the active ones)
    nodes::Vector{Int}   # the ids of their nodes, ascending: device node k is model node nodes[k]
end

function check(m::Union{GPUModel,Nothing}, rc::Integer)
    rc == 0 && return nothing
    buf = zeros(UInt8, 1024)
    if m === nothing
        msg = unsafe_string(ccall((:amr_create_error, LIB), Cstring, ()))
    else
        ccall((:amr_last_error, LIB), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), m.h, buf, length(buf))
        msg = unsafe_string(pointer(buf))
    end
    return Amaru.failure("libamaru_gpu ($rc): $msg")
end

material_code(m::LinearElastic) = (Int32(0), [m.E, m.ν, 0, 0, 0, 0, 0, 0])
material_code(m::VonMises) = (Int32(1), [m.E, m.ν, m.σy, m.H, 0, 0, 0, 0])
material_code(m::DruckerPrager) = (Int32(2), [m.E, m.ν, m.α, m.κ, m.H, 0, 0, 0])
# the linear elastic skeletons of the coupled elements (their fluid / thermal parameters go to the mount)
material_code(m::LinearElasticSeep) = (Int32(0), [m.E, m.ν, 0, 0, 0, 0, 0, 0])
material_code(m::LinearElasticThermo) = (Int32(0), [m.E, m.ν, 0, 0, 0, 0, 0, 0])
material_code(m) = error("AmaruGPU: material $(typeof(m)) is not on the GPU path")

"""
    activate!(model, stage)

Applies `stage.toactivate` as mech_stage_solver! does (src/mech/mech-solver.jl:216-220).  The device
model holds the active elements and their nodes (gpu_model!), so the stage assembles and updates only
the active elements and configure_dofs! numbers only their nodes (src/bc.jl:200-203).
"""
function activate!(model::FEModel, stage::Stage)
    for elem in stage.toactivate
        elem.active = true
    end
    return nothing
end

"""
    GPUModel(model::FEModel; elems=model.elems)

Creates the device model over `elems` and the nodes they use: nodes, MechSolid elements with their
material parameters and quadrature, pattern and contribution map (amr_model_create).
"""
function GPUModel(model::FEModel; elems=model.elems)
    all(e -> e isa MechSolid || e isa HMSolid || e isa TMSolid, elems) ||
        error("AmaruGPU: only MechSolid, HMSolid and TMSolid elements are on the GPU path")
    ids = sort(unique([n.id for e in elems for n in e.nodes]))
    loc = Dict(id => k - 1 for (k, id) in enumerate(ids))
    nnodes = length(ids)
    coords = zeros(3, nnodes)
    for (k, id) in enumerate(ids)
        n = model.nodes[id]
        coords[:, k] .= (n.coord.x, n.coord.y, n.coord.z)
    end
    nel = length(elems)
    shape = Int32[SHAPES[e.shape.name] for e in elems]
    nips = Int32[length(e.ips) for e in elems]
    conn_ptr = zeros(Int64, nel + 1)
    conn = Int64[]
    mat_type = zeros(Int32, nel)
    mat_params = zeros(8, nel)
    for (k, e) in enumerate(elems)
        append!(conn, [loc[n.id] for n in e.nodes])
        conn_ptr[k+1] = length(conn)
        t, p = material_code(e.mat)
        mat_type[k] = t
        mat_params[:, k] .= p
    end
    ctx = model.ctx
    GC.@preserve coords shape nips conn_ptr conn mat_type mat_params begin
        d = ModelDesc(ctx.ndim, STRESSMODELS[ctx.stressmodel], ctx.thickness, nnodes, pointer(coords), nel,
                      pointer(shape), pointer(nips), pointer(conn_ptr), pointer(conn), pointer(mat_type),
                      pointer(mat_params))
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:amr_model_create, LIB), Cint, (Ref{ModelDesc}, Ref{Ptr{Cvoid}}), d, h)
        st = check(nothing, rc)
        st === nothing || error(st.message)
    end
    g = GPUModel(h[], 0, 0, collect(Any, elems), ids)
    finalizer(release!, g)
    return g
end

function release!(g::GPUModel)
    g.h == C_NULL || ccall((:amr_model_destroy, LIB), Cint, (Ptr{Cvoid},), g.h)
    g.h = C_NULL
    return nothing
end

"""
    gpu_model!(model) -> GPUModel

The model's device handle over its active elements: kept while the active set stays, rebuilt when a
stage's toactivate changed it.  A new handle takes the IP states of the elements' IpState objects
(where sync_states! left the last stage's), so the states move with their elements.
"""
function gpu_model!(model::FEModel)
    act = [e for e in model.elems if e.active]
    g = get(GPU_MODELS, objectid(model), nothing)
    if g === nothing || length(g.elems) != length(act) || any(a !== b for (a, b) in zip(g.elems, act))
        g === nothing || release!(g)
        g = GPUModel(model; elems=act)
        load_states!(g)
        GPU_MODELS[objectid(model)] = g
    end
    return g
end

# the IpState objects of g's elements into the device (the inverse of sync_states!)
function load_states!(g::GPUModel)
    S = zeros(16, sum(length(e.ips) for e in g.elems; init=0))
    k = 0
    for elem in g.elems, ip in elem.ips
        k += 1
        st = ip.state
        S[1:6, k] .= st.σ
        S[7:12, k] .= st.ε
        hasfield(typeof(st), :εpa) && (S[13, k] = st.εpa)
        hasfield(typeof(st), :Δλ) && (S[14, k] = st.Δλ)
        hasfield(typeof(st), :Δγ) && (S[14, k] = st.Δγ)
    end
    set_state!(g, S)
    return g
end

# fn(handle over every element of the model, holding the IpState objects' states): output covers every
# element, as update_output_data! does (src/fe-model.jl:341-427)
function with_all_elements(fn, model::FEModel)
    g = GPU_MODELS[objectid(model)]
    length(g.elems) == length(model.elems) && return fn(g)
    full = GPUModel(model)
    try
        load_states!(full)
        return fn(full)
    finally
        release!(full)
    end
end

"""
    set_dofs!(g, model, dofs, nu)

Passes the numbering of configure_dofs! (src/bc.jl:198-233) to the library.
"""
function set_dofs!(g::GPUModel, model::FEModel, dofs, nu)
    eq = fill(Int64(-1), 3, length(g.nodes))
    keys = (:ux, :uy, :uz)
    for (i, id) in enumerate(g.nodes)
        n = model.nodes[id]
        for (k, key) in enumerate(keys)
            haskey(n.dofdict, key) && (eq[k, i] = n.dofdict[key].eq_id - 1)
        end
    end
    rc = ccall((:amr_set_dofs, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Int64, Int64), g.h, eq, length(dofs), nu)
    st = check(g, rc)
    st === nothing || error(st.message)
    g.ndofs, g.nu = length(dofs), nu
    return g
end

"""
    mount_K(g)

mount_K on the device; returns K as a SparseMatrixCSC in the reference's
layout (1-based), with its stored-entry pattern (amr_get_K_csc).
"""
function mount_K(g::GPUModel; reference_order::Bool=true)
    ccall((:amr_set_assembly, LIB), Cint, (Ptr{Cvoid}, Int32), g.h, reference_order ? 1 : 0)
    st = check(g, ccall((:amr_assemble_K, LIB), Cint, (Ptr{Cvoid},), g.h))
    st === nothing || error(st.message)
    nnz = Ref{Int64}(0)
    ccall((:amr_get_K_nnz, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}), g.h, nnz)
    colptr = zeros(Int64, g.ndofs + 1)
    rowval = zeros(Int64, nnz[])
    nzval = zeros(nnz[])
    st = check(g, ccall((:amr_get_K_csc, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}),
                        g.h, colptr, rowval, nzval))
    st === nothing || error(st.message)
    ccall((:amr_set_assembly, LIB), Cint, (Ptr{Cvoid}, Int32), g.h, 0)
    return SparseMatrixCSC(g.ndofs, g.ndofs, colptr .+ 1, rowval .+ 1, nzval)
end

"""
    set_amg_smoothing!(g, on::Bool)

Smoothed-aggregation prolongators (true, the default) or the tentative ones
(false) for the multigrid solves of `g` (amr_set_amg_smoothing).
"""
function set_amg_smoothing!(g::GPUModel, on::Bool)
    st = check(g, ccall((:amr_set_amg_smoothing, LIB), Cint, (Ptr{Cvoid}, Int32), g.h, on ? 1 : 0))
    st === nothing || error(st.message)
    return g
end

"""
    update_state!(g, dU) -> (dFin, status)

update_state!(elems, dU, t) on the device (trial states from the committed ones).
"""
function update_state!(g::GPUModel, dU::Vector{Float64})
    dF = zeros(g.ndofs)
    rc = ccall((:amr_update_state, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), g.h, dU, dF)
    st = check(g, rc)
    return dF, st === nothing ? Amaru.success() : st
end

"""
    solve_system!(g, U, F; rtol=1e-8) -> status

solve_system! on the last assembled K: U[1:nu] and F[nu+1:end] are filled.
"""
function solve_system!(g::GPUModel, U::Vector{Float64}, F::Vector{Float64}; rtol=1e-8, method=0)
    opts = SolveOpts(method, rtol, 20000, 32)
    stats = Ref(SolveStats(0, 0, 0.0, 0.0))
    rc = ccall((:amr_solve, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{SolveOpts}, Ref{SolveStats}),
               g.h, U, F, opts, stats)
    st = check(g, rc)
    return st === nothing ? Amaru.success() : st
end

# After every converged increment of a device stage (amr_set_increment_callback): the dof values so far,
# the committed IP states, sctx.T / inc / out, then update_records!(ana, checkpoint=...) as
# mech_stage_solver! calls it (src/mech/mech-solver.jl:394-424).  A failed update_records! stops the stage.
mutable struct IncrementContext
    ana::MechAnalysis
    g::GPUModel
    dofs::Vector{Amaru.Dof}
    base_u::Vector{Float64}
    base_f::Vector{Float64}
end

struct IncrementInfo
    T::Float64; increment::Int32; checkpoint::Int32; ndofs::Int64
    U::Ptr{Float64}; F::Ptr{Float64}
end

function increment_hook(user::Ptr{Cvoid}, info::Ptr{IncrementInfo})::Cint
    try
        ctx = unsafe_pointer_to_objref(user)::IncrementContext
        i = unsafe_load(info)
        U = unsafe_wrap(Array, i.U, i.ndofs)
        F = unsafe_wrap(Array, i.F, i.ndofs)
        for (k, dof) in enumerate(ctx.dofs)
            dof.vals[dof.name] = ctx.base_u[k] + U[k]
            dof.vals[dof.natname] = ctx.base_f[k] + F[k]
        end
        sync_states!(ctx.g, ctx.ana.model)
        sctx = ctx.ana.sctx
        sctx.T = i.T
        sctx.inc = i.increment
        i.checkpoint != 0 && (sctx.out += 1)
        st = Amaru.update_records!(ctx.ana, checkpoint=i.checkpoint != 0)
        return Amaru.failed(st) ? Cint(1) : Cint(0)
    catch
        return Cint(1)  # no Julia exception crosses the C ABI: the stage stops
    end
end

"""
    gpu_stage_solver!(ana::MechAnalysis, stage::Stage; args...)

mech_stage_solver! with the Newton loop, K, the solves and the IP states on
the device.  The essential values and loads come from Amaru's own
configure_dofs! and get_bc_vals.  After every converged increment the library
calls back into Julia, where the dof values are updated as the reference
does (src/mech/mech-solver.jl:394-397), the IP states are copied into the
elements' IpState objects, and update_records! runs with the reference's
checkpoint flag and output numbering (:410-424): every checkpoint of nouts gets
its record, and the loggers and monitors see every increment.  Stage 1 writes
its initial record first (:234-242), and a failed stage its last one (:488).
"""
function gpu_stage_solver!(ana::MechAnalysis, stage::Stage; args...)
    args = NamedTuple(args)
    model = ana.model
    activate!(model, stage)
    g = gpu_model!(model)
    dofs, nu = Amaru.configure_dofs!(model, stage.bcs)
    model.ndofs = length(dofs)
    set_dofs!(g, model, dofs, nu)
    if stage.id == 1
        for dof in dofs
            dof.vals[dof.name] = 0.0
            dof.vals[dof.natname] = 0.0
        end
        Amaru.update_records!(ana, force=true)
    end
    Uex, Fex = Amaru.get_bc_vals(model, stage.bcs)
    scheme = Dict(:FE => 0, :ME => 1, :BE => 2, :Ralston => 3)[Symbol(args.scheme)]
    lin = SolveOpts(LINEAR_METHOD[], 1e-8, 20000, 32)
    p = StageParams(args.tol, args.rtol, args.rspan, args.dT0, args.dTmin, args.dTmax, scheme, args.maxits,
                    args.autoinc, stage.nincs, stage.nouts, lin)
    U = zeros(length(dofs))
    F = zeros(length(dofs))
    stats = StageStats()
    ctx = IncrementContext(ana, g, dofs, [dof.vals[dof.name] for dof in dofs], [dof.vals[dof.natname] for dof in dofs])
    hook = @cfunction(increment_hook, Cint, (Ptr{Cvoid}, Ptr{IncrementInfo}))
    rc = GC.@preserve ctx begin
        ccall((:amr_set_increment_callback, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
              g.h, hook, pointer_from_objref(ctx))
        r = ccall((:amr_stage_run, LIB), Cint,
                  (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{StageParams}, Ptr{Float64}, Ptr{Float64},
                   Ref{StageStats}), g.h, Uex, Fex, p, U, F, stats)
        ccall((:amr_set_increment_callback, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), g.h, C_NULL, C_NULL)
        r
    end
    if rc == 0 || rc == -11
        for (i, dof) in enumerate(dofs)  # the converged increments' values (as the last callback set them)
            dof.vals[dof.name] = ctx.base_u[i] + U[i]
            dof.vals[dof.natname] = ctx.base_f[i] + F[i]
        end
        sync_states!(g, model)
    end
    rc == 0 && return Amaru.success()
    st = check(g, rc)
    rc == -11 && Amaru.update_records!(ana, force=true)
    return st
end

"""
    sync_states!(g, model)

Copies the device IP states into the IpState objects of the model's elements, in
element and IP order: σ and ε, and for the plastic materials εpa and Δλ (Δγ of
DruckerPragerState).  Julia code that reads ip.state after a GPU stage, such as
update_output_data!'s element values and the loggers, then sees the stage's
result.
"""
sync_states!(g::GPUModel, model::FEModel) = (copy_states!(get_state(g), g.elems); model)

# S (16 x nip, element and IP order of the models one after the other) into the IpState objects
copy_states!(S::Matrix{Float64}, models::Union{Tuple,AbstractVector{<:FEModel}}) =
    copy_states!(S, [elem for model in models for elem in model.elems])

function copy_states!(S::Matrix{Float64}, elems::AbstractVector)
    k = 0
    for elem in elems, ip in elem.ips
        k += 1
        st = ip.state
        st.σ = typeof(st.σ)(view(S, 1:6, k))
        st.ε = typeof(st.ε)(view(S, 7:12, k))
        hasfield(typeof(st), :εpa) && (st.εpa = S[13, k])
        hasfield(typeof(st), :Δλ) && (st.Δλ = S[14, k])
        hasfield(typeof(st), :Δγ) && (st.Δγ = S[14, k])
    end
    k == size(S, 2) || error("AmaruGPU: IP count differs from the device model's")
    return nothing
end

const GPU_MODELS = Dict{UInt,GPUModel}()

# linear method of the stage solver: 0 block-Jacobi, 2 aggregation multigrid (amr_solve_opts.method)
const LINEAR_METHOD = Ref{Int32}(2)

"""
    solve_gpu!(ana::MechAnalysis; linear=:amg, args...)

solve! with the stage solver replaced by gpu_stage_solver!; `linear` picks the
preconditioner of the FP32 PCG (:amg multigrid or :jacobi block-Jacobi).
"""
function solve_gpu!(ana::MechAnalysis; linear::Symbol=:amg, args...)
    LINEAR_METHOD[] = linear === :jacobi ? Int32(0) : Int32(2)
    args = Amaru.checkargs(args, Amaru.mech_solver_params)
    return Amaru.stage_iterator!(gpu_stage_solver!, ana; args...)
end

# ---------------------------------------------------------------------------
# Dynamic analyses: dyn_stage_solver! (src/mech/dyn-solver.jl:203-534) on the device.
# ---------------------------------------------------------------------------
struct DynParams
    tol::Float64; dTmin::Float64; dTmax::Float64; rspan::Float64
    alpha::Float64; beta::Float64; tspan::Float64
    maxits::Int32; autoinc::Int32; nincs::Int32; nouts::Int32
    linear::SolveOpts
    sism::Int32; sism_dir::Int32
    tss::Float64; tds::Float64
    sism_acc::Ptr{Float64}; sism_n::Int64
end

# component of a seismic direction key (node.dofdict holds both the dof name and its natural name)
const SISM_DIRS = Dict(:ux => 0, :fx => 0, :uy => 1, :fy => 1, :uz => 2, :fz => 2)

"""
    gpu_dyn_stage_solver!(ana::Amaru.DynamicAnalysis, stage::Stage; args...)

dyn_stage_solver! of a first stage with K, M, the solves and the IP states on the
device.  Boundary values come from Amaru's get_bc_vals at t = 0 and t = 1 (they must
be affine in t); ux/fx/vx/ax land in dof.vals as the reference writes them
(src/mech/dyn-solver.jl:420-425).  The IP states are copied into the IpState
objects and the record of the stage's last checkpoint (or of its failure) is
written; the initial record (:299-300) and those of intermediate checkpoints are
not, as the increments run on the device.
"""
function gpu_dyn_stage_solver!(ana::Amaru.DynamicAnalysis, stage::Stage; args...)
    args = NamedTuple(args)
    model = ana.model
    activate!(model, stage)
    g = gpu_model!(model)
    dofs, nu = Amaru.configure_dofs!(model, stage.bcs)
    model.ndofs = length(dofs)
    set_dofs!(g, model, dofs, nu)
    rho = Float64[ elem.props.ρ for elem in g.elems ]
    check(g, ccall((:amr_set_density, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, rho))
    U0, F0 = Amaru.get_bc_vals(model, stage.bcs, 0.0)
    U1, F1 = Amaru.get_bc_vals(model, stage.bcs, 1.0)
    lin = SolveOpts(LINEAR_METHOD[], 1e-8, 20000, 32)
    # seismic input: the record of sism_file (readdlm, times 9.81, row by row, as sismic_force reads it)
    sism = get(args, :sism, false)
    acc = sism ? vec(permutedims(9.81 .* readdlm(args.sism_file))) : Float64[]
    p = DynParams(args.tol, args.dTmin, args.dTmax, args.rspan, args.alpha, args.beta, stage.tspan,
                  args.maxits, args.autoinc, stage.nincs, stage.nouts, lin,
                  Int32(sism), Int32(get(SISM_DIRS, Symbol(get(args, :sism_dir, "fx")), 0)),
                  get(args, :tss, 0.0), get(args, :tds, 0.0), pointer(acc), Int64(length(acc)))
    n = length(dofs)
    U, V, A, F = zeros(n), zeros(n), zeros(n), zeros(n)
    stats = StageStats()
    rc = GC.@preserve acc ccall((:amr_dyn_stage_run, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{DynParams},
                Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{StageStats}),
               g.h, U0, U1 .- U0, F0, F1 .- F0, p, U, V, A, F, stats)
    if rc == 0 || rc == -11
        keys = Dict(:ux => (:ux, :fx, :vx, :ax), :uy => (:uy, :fy, :vy, :ay), :uz => (:uz, :fz, :vz, :az))
        for (i, dof) in enumerate(dofs)
            us, fs, vs, as = keys[dof.name]
            dof.vals[us] = U[i]; dof.vals[fs] = F[i]; dof.vals[vs] = V[i]; dof.vals[as] = A[i]
        end
        # IP states into the IpState objects; the record of the last checkpoint (dyn-solver.jl:447-480)
        # or of the failure (:532), with the stage's time as the reference keeps it
        sync_states!(g, model)
        ana.sctx.T = stats.T
        ana.sctx.t = stats.T * stage.tspan
    end
    if rc == 0
        ana.sctx.out += max(stage.nouts, 1)
        Amaru.update_records!(ana, checkpoint=true)
        return Amaru.success()
    end
    st = check(g, rc)
    rc == -11 && Amaru.update_records!(ana, force=true)
    return st
end

"""
    solve_gpu!(ana::Amaru.DynamicAnalysis; linear=:amg, args...)

solve! of a dynamic analysis (dyn_solver_params) with gpu_dyn_stage_solver!.
"""
function solve_gpu!(ana::Amaru.DynamicAnalysis; linear::Symbol=:amg, args...)
    LINEAR_METHOD[] = linear === :jacobi ? Int32(0) : Int32(2)
    args = Amaru.checkargs(args, Amaru.dyn_solver_params)
    return Amaru.stage_iterator!(gpu_dyn_stage_solver!, ana; args...)
end

# ---------------------------------------------------------------------------
# VTU output: save_vtu (src/mesh/io.jl:167-274, ascii) written by the library.
# ---------------------------------------------------------------------------
struct VtuArray
    name::Cstring; type::Int32; ncomp::Int32; on_device::Int32; pad::Int32; data::Ptr{Cvoid}
end
const VTU_TYPES = Dict(Float64 => Int32(0), Int32 => Int32(1), Int64 => Int32(2), UInt64 => Int32(3))

"""
    save_gpu(model::FEModel, filename::String; compress=false)

save(model, filename; compress) for .vtu files: update_output_data!(model), the tag fields save_vtu adds
(src/mesh/io.jl:168-192, with Amaru's own encoders and the same Set order), then the file written by
amr_write_vtu (ascii) or amr_write_vtu_compressed (zlib blocks appended) from model.node_data and
model.elem_data, byte for byte as save_vtu writes it.
"""
function save_gpu(model::FEModel, filename::String; compress::Bool=false)
    Amaru.update_output_data!(model)
    tags = collect(Set(elem.tag for elem in model.elems))
    if length(tags) > 1 || tags[1] != ""
        tag_d = Dict(tag => i for (i, tag) in enumerate(tags))
        parts = Tuple{String,String}[]
        for tag in tags
            length(codeunits(tag)) > 16 && error("Mesh: tag '$tag' too long. Max length is 16 UTF units.")
            push!(parts, Amaru.safe_string_cut(tag, 8))
        end
        model.elem_data["tag-s1"] = UInt64[Amaru.encode_string_to_uint64(parts[tag_d[e.tag]][1]) for e in model.elems]
        model.elem_data["tag-s2"] = UInt64[Amaru.encode_string_to_uint64(parts[tag_d[e.tag]][2]) for e in model.elems]
        model.elem_data["tag"] = Int[tag_d[e.tag] - 1 for e in model.elems]
    end
    keep = Any[]
    function arrays(d)
        out = VtuArray[]
        for (name, a) in d
            isempty(a) && continue
            a = haskey(VTU_TYPES, eltype(a)) ? a : Float64.(a)
            push!(keep, a, name)
            push!(out, VtuArray(Base.unsafe_convert(Cstring, name), VTU_TYPES[eltype(a)], Int32(size(a, 2)),
                                Int32(0), Int32(0), pointer(a)))
        end
        return out
    end
    pd, cd = arrays(model.node_data), arrays(model.elem_data)
    with_all_elements(model) do g
        GC.@preserve keep begin
            rc = compress ?
                ccall((:amr_write_vtu_compressed, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{VtuArray}, Int32,
                      Ptr{VtuArray}, Int32, Int32), g.h, filename, pd, length(pd), cd, length(cd), Int32(0)) :
                ccall((:amr_write_vtu, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{VtuArray}, Int32, Ptr{VtuArray},
                      Int32, Int32), g.h, filename, pd, length(pd), cd, length(cd), Int32(0))
            check(g, rc)
        end
    end
    return nothing
end

# ---------------------------------------------------------------------------
# Modal analyses: mech_modal_solver! (src/mech/mech-modal-solver.jl:72-235) on the device.
# ---------------------------------------------------------------------------
struct ModalParams
    nmodes::Int32; max_iters::Int32; tol::Float64
end
mutable struct ModalStats
    iterations::Int32; block::Int32; max_residual::Float64; seconds::Float64
    ModalStats() = new(0, 0, 0.0, 0.0)
end

"""
    gpu_modal_solver!(ana::MechModalAnalysis, stage::Stage; nmodes=5, args...)

ana.freqs (omega, ascending) and ana.modes (P's unit eigenvectors on the unknown DOFs) of
mech_modal_solver!, computed on the device.
"""
function gpu_modal_solver!(ana::MechModalAnalysis, stage::Stage; nmodes::Integer=5, args...)
    model = ana.model
    activate!(model, stage)
    g = gpu_model!(model)
    dofs, nu = Amaru.configure_dofs!(model, stage.bcs)
    model.ndofs = length(dofs)
    set_dofs!(g, model, dofs, nu)
    rho = Float64[ elem.props.ρ for elem in g.elems ]
    check(g, ccall((:amr_set_density, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, rho))
    w = zeros(nmodes)
    V = zeros(nu, nmodes)
    st = ModalStats()
    check(g, ccall((:amr_modal_run, LIB), Cint, (Ptr{Cvoid}, Ref{ModalParams}, Ptr{Float64}, Ptr{Float64},
                   Ref{ModalStats}), g.h, ModalParams(nmodes, 1000, 1e-7), w, V, st))
    ana.freqs = w
    ana.modes = V
    if get(args, :rayleigh, false)
        # the rayleigh option (src/mech/mech-modal-solver.jl:204-226): two damping ratios and two of the
        # computed modes, read from standard input in the reference's order
        ask(q) = (println(q); chomp(readline()))
        ξ1 = parse(Float64, ask("Damping ratio 1 (xi1 = c/c_c)?"))
        ξ2 = parse(Float64, ask("Damping ratio 2 (xi2 = c/c_c)?"))
        i1 = parse(Int, ask("Mode of the first frequency?"))
        i2 = parse(Int, ask("Mode of the second frequency?"))
        α, β = rayleigh_coefficients(w[i1], w[i2], ξ1, ξ2)
        Amaru.info("Rayleigh alpha: ", α)
        Amaru.info("Rayleigh beta:", β)
    end
    return Amaru.success()
end

"""
    rayleigh_coefficients(w1, w2, ξ1, ξ2) -> (α, β)

Rayleigh damping C = αM + βK whose damping ratio α/(2ω) + βω/2 is ξ1 at ω = w1 and ξ2 at ω = w2
(src/mech/mech-modal-solver.jl:221-222).
"""
function rayleigh_coefficients(w1, w2, ξ1, ξ2)
    d = w1^2 - w2^2
    return 2 * (w1^2 * w2 * ξ2 - w1 * w2^2 * ξ1) / d, 2 * (w1 * ξ1 - w2 * ξ2) / d
end

# ---------------------------------------------------------------------------
# Output data: nodal_patch_recovery (src/fe-model.jl:504-702) on the device.
# ---------------------------------------------------------------------------
const FIELD_SYMBOLS = [:σxx, :σyy, :σzz, :σyz, :σxz, :σxy, :σvm, :σ1, :σ2, :σ3,
                       :εxx, :εyy, :εzz, :εyz, :εxz, :εxy, :ep, :epa, :j1, :srj2d]
# the keys the same codes carry in an axisymmetric analysis (src/tools/tensors.jl:182-193)
const AXI_FIELD_SYMBOLS = [:σrr, :σyy, :σtt, :σyz, :σxz, :σry, :σvm, :σ1, :σ2, :σ3,
                           :εrr, :εyy, :εtt, :εyz, :εxz, :εry, :ep, :epa, :j1, :srj2d]

"""
    nodal_patch_recovery_gpu(model::FEModel)

The `(V_rec, fields)` pair of nodal_patch_recovery(model), from the IP states the
model's GPU handle holds (the last gpu_stage_solver! stage).
"""
function nodal_patch_recovery_gpu(model::FEModel)
    with_all_elements(model) do g
        n = Ref{Int32}(0)
        codes = zeros(Int32, length(FIELD_SYMBOLS))
        check(g, ccall((:amr_recovery_fields, LIB), Cint, (Ptr{Cvoid}, Ptr{Int32}, Int32, Ref{Int32}),
                       g.h, codes, Int32(length(codes)), n))
        V = zeros(length(model.nodes), n[])  # a handle over every element holds every used node
        n[] > 0 && check(g, ccall((:amr_recover_nodal, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, V))
        syms = model.ctx.stressmodel == :axisymmetric ? AXI_FIELD_SYMBOLS : FIELD_SYMBOLS
        return V, syms[codes[1:n[]] .+ 1]
    end
end

# GPU-backed model?  update_output_data! picks the recovery with it (the one-line hook at
# src/fe-model.jl:379: V_rec, fields_rec = has_gpu(model) ? nodal_patch_recovery_gpu(model) :
# nodal_patch_recovery(model)); redefining nodal_patch_recovery(::FEModel) here would replace
# the CPU method for every model.
has_gpu(model::FEModel) = haskey(GPU_MODELS, objectid(model))

# ---------------------------------------------------------------------------
# Batches: independent models joined into one handle (amr_set_parts), each
# running its own mech_stage_solver! with one kernel launch per step for all.
# ---------------------------------------------------------------------------
function model_arrays(model::FEModel)
    elems = model.elems
    all(e -> e isa MechSolid || e isa HMSolid || e isa TMSolid, elems) ||
        error("AmaruGPU: only MechSolid, HMSolid and TMSolid elements are on the GPU path")
    all(e -> e.active, elems) || error("AmaruGPU: batched and served models must have every element active")
    coords = zeros(3, length(model.nodes))
    for (i, n) in enumerate(model.nodes)
        coords[:, i] .= (n.coord.x, n.coord.y, n.coord.z)
    end
    nel = length(elems)
    conn_ptr = zeros(Int64, nel + 1); conn = Int64[]
    mat_type = zeros(Int32, nel); mat_params = zeros(8, nel)
    for (k, e) in enumerate(elems)
        append!(conn, [n.id - 1 for n in e.nodes])
        conn_ptr[k+1] = length(conn)
        mat_type[k], mat_params[:, k] = material_code(e.mat)
    end
    shape = Int32[SHAPES[e.shape.name] for e in elems]
    nips = Int32[length(e.ips) for e in elems]
    return coords, shape, nips, conn_ptr, conn, mat_type, mat_params
end

function eq_array(model::FEModel)
    eq = fill(Int64(-1), 3, length(model.nodes))
    for n in model.nodes, (k, key) in enumerate((:ux, :uy, :uz))
        haskey(n.dofdict, key) && (eq[k, n.id] = n.dofdict[key].eq_id - 1)
    end
    return eq
end

# immutable mirror of amr_stage_stats, for arrays and for embedding in other records
struct PartStats
    status::Int32; increments::Int32; iterations::Int32; krylov_iterations::Int32
    residue::Float64; T::Float64; seconds::Float64; solve_seconds::Float64
end

mutable struct GPUBatch
    h::Ptr{Cvoid}
    models::Vector{FEModel}
    node_ptr::Vector{Int64}
end

"""
    GPUBatch(models)

Joins independent models (same ndim, stress model and thickness) into one device
model, model i's nodes and elements after those of models 1..i-1, and declares
each a part: the batched solver and stage driver then run every model as if it
were alone.
"""
function GPUBatch(models::Vector{<:FEModel})
    parts = [model_arrays(m) for m in models]
    node_ptr = cumsum([0; [size(p[1], 2) for p in parts]])
    coords = reduce(hcat, [p[1] for p in parts])
    shape = reduce(vcat, [p[2] for p in parts]); nips = reduce(vcat, [p[3] for p in parts])
    conn = reduce(vcat, [p[5] .+ node_ptr[i] for (i, p) in enumerate(parts)])
    conn_ptr = cumsum([0; reduce(vcat, [diff(p[4]) for p in parts])])
    mat_type = reduce(vcat, [p[6] for p in parts]); mat_params = reduce(hcat, [p[7] for p in parts])
    ctx = models[1].ctx
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve coords shape nips conn_ptr conn mat_type mat_params begin
        d = ModelDesc(ctx.ndim, STRESSMODELS[ctx.stressmodel], ctx.thickness, size(coords, 2), pointer(coords),
                      length(shape), pointer(shape), pointer(nips), pointer(conn_ptr), pointer(conn),
                      pointer(mat_type), pointer(mat_params))
        st = check(nothing, ccall((:amr_model_create, LIB), Cint, (Ref{ModelDesc}, Ref{Ptr{Cvoid}}), d, h))
        st === nothing || error(st.message)
    end
    b = GPUBatch(h[], collect(models), node_ptr)
    finalizer(x -> ccall((:amr_model_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), b)
    rc = ccall((:amr_set_parts, LIB), Cint, (Ptr{Cvoid}, Int64, Ptr{Int64}), b.h, length(models), node_ptr)
    rc == 0 || error("amr_set_parts failed ($rc)")
    return b
end

"""
    solve_batch!(b, stages; linear=:amg, args...)

One stage per model (stages[i] for models[i]), run together: each model's DOFs are
numbered by Amaru's configure_dofs! and its loads taken from get_bc_vals; the
joined numbering puts every model's unknowns first.  `linear` picks the per-part
PCG's preconditioner: the joined model's multigrid V-cycle (:amg) or block-Jacobi
in one persistent launch (:jacobi).  Updates each model's dof values as
mech_stage_solver! does and returns one status per model.
"""
function solve_batch!(b::GPUBatch, stages::Vector{Stage}; linear::Symbol=:amg, args...)
    args = Amaru.checkargs(args, Amaru.mech_solver_params)
    eqs, Us, Fs, nus, nds, dofss = [], [], [], Int[], Int[], []
    for (m, st) in zip(b.models, stages)
        activate!(m, st)
        all(e -> e.active, m.elems) || error("AmaruGPU: batched models must have every element active")
        dofs, nu = Amaru.configure_dofs!(m, st.bcs)
        m.ndofs = length(dofs)
        Uex, Fex = Amaru.get_bc_vals(m, st.bcs)
        push!(eqs, eq_array(m)); push!(Us, Uex); push!(Fs, Fex); push!(nus, nu); push!(nds, length(dofs))
        push!(dofss, dofs)
    end
    NU, ND = sum(nus), sum(nds)
    offU = cumsum([0; nus[1:end-1]]); offP = cumsum([0; (nds .- nus)[1:end-1]])
    joined(i, e) = e < 0 ? e : (e < nus[i] ? offU[i] + e : NU + offP[i] + (e - nus[i]))
    eq = reduce(hcat, [map(e -> joined(i, e), eqs[i]) for i in eachindex(eqs)])
    Uex = zeros(ND); Fex = zeros(ND)
    for i in eachindex(eqs), e in 0:nds[i]-1
        Uex[joined(i, e)+1] = Us[i][e+1]; Fex[joined(i, e)+1] = Fs[i][e+1]
    end
    ccall((:amr_set_dofs, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Int64, Int64), b.h, eq, ND, NU)
    scheme = Dict(:FE => 0, :ME => 1, :BE => 2, :Ralston => 3)[Symbol(args.scheme)]
    method = linear === :jacobi ? Int32(0) : Int32(2)  # per-part block-Jacobi, or the joined multigrid
    p = StageParams(args.tol, args.rtol, args.rspan, args.dT0, args.dTmin, args.dTmax, scheme, args.maxits,
                    args.autoinc, stages[1].nincs, stages[1].nouts, SolveOpts(method, 1e-8, 20000, 32))
    U = zeros(ND); F = zeros(ND); stats = StageStats()
    ccall((:amr_stage_run, LIB), Cint,
          (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{StageParams}, Ptr{Float64}, Ptr{Float64}, Ref{StageStats}),
          b.h, Uex, Fex, p, U, F, stats)
    buf = Vector{PartStats}(undef, length(b.models))
    ccall((:amr_get_part_stats, LIB), Cint, (Ptr{Cvoid}, Int64, Ptr{PartStats}), b.h, length(b.models), buf)
    for i in eachindex(b.models), (e, dof) in enumerate(dofss[i])
        j = joined(i, e - 1) + 1
        dof.vals[dof.name] += U[j]
        dof.vals[dof.natname] += F[j]
    end
    # every part's IP states into its IpState objects (the parts' elements follow one another)
    S = zeros(16, sum(length(e.ips) for m in b.models for e in m.elems))
    rc = ccall((:amr_get_state, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), b.h, S)
    rc == 0 || error("amr_get_state failed ($rc)")
    copy_states!(S, b.models)
    return [s.status == 0 ? Amaru.success() : Amaru.failure("Solver did not converge.") for s in buf]
end

# ---------------------------------------------------------------------------
# Serving: stages of independent models submitted as they arrive (amr_server_*).
# ---------------------------------------------------------------------------
struct Request
    model::ModelDesc
    eq_id::Ptr{Int64}; ndofs::Int64; nu::Int64
    Uex::Ptr{Float64}; Fex::Ptr{Float64}
    loads::Ptr{Cvoid}; nloads::Int32; pad::Int32
    stage::StageParams
end

mutable struct RequestResult
    status::Int32; active_at_admit::Int32; bytes::Int64
    t_submit::Float64; t_admit::Float64; t_done::Float64
    stage::PartStats
    t_stage::Float64; dev_start::Float64; dev_end::Float64
    RequestResult() = new(0, 0, 0, 0.0, 0.0, 0.0, PartStats(0, 0, 0, 0, 0.0, 0.0, 0.0, 0.0), 0.0, 0.0, 0.0)
end

struct ServerConfig
    hbm_budget_bytes::Float64
    max_active::Int32
    pad::Int32
end

mutable struct GPUServer
    h::Ptr{Cvoid}
    pending::Dict{Int64,Tuple{FEModel,Any}}
end

"""
    GPUServer(hbm_budget_bytes; max_active=4)

A request loop on the current GPU: up to max_active requests on the device at
once, admitted in arrival order as slots and memory free up.
"""
function GPUServer(budget; max_active::Integer=4)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:amr_server_create, LIB), Cint, (Ref{ServerConfig}, Ref{Ptr{Cvoid}}),
               ServerConfig(Float64(budget), Int32(max_active), 0), h)
    rc == 0 || error("amr_server_create failed ($rc)")
    s = GPUServer(h[], Dict{Int64,Tuple{FEModel,Any}}())
    finalizer(x -> ccall((:amr_server_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), s)
    return s
end

"""
    submit!(srv, model, stage; args...) -> id

Queues one stage of `model` (solve! keyword arguments); the server copies it.
"""
function submit!(srv::GPUServer, model::FEModel, stage::Stage; args...)
    args = Amaru.checkargs(args, Amaru.mech_solver_params)
    activate!(model, stage)
    dofs, nu = Amaru.configure_dofs!(model, stage.bcs)
    model.ndofs = length(dofs)
    Uex, Fex = Amaru.get_bc_vals(model, stage.bcs)
    coords, shape, nips, conn_ptr, conn, mat_type, mat_params = model_arrays(model)
    eq = eq_array(model)
    ctx = model.ctx
    scheme = Dict(:FE => 0, :ME => 1, :BE => 2, :Ralston => 3)[Symbol(args.scheme)]
    p = StageParams(args.tol, args.rtol, args.rspan, args.dT0, args.dTmin, args.dTmax, scheme, args.maxits,
                    args.autoinc, stage.nincs, stage.nouts, SolveOpts(0, 1e-8, 20000, 32))
    id = Ref{Int64}(0)
    GC.@preserve coords shape nips conn_ptr conn mat_type mat_params eq Uex Fex begin
        d = ModelDesc(ctx.ndim, STRESSMODELS[ctx.stressmodel], ctx.thickness, size(coords, 2), pointer(coords),
                      length(shape), pointer(shape), pointer(nips), pointer(conn_ptr), pointer(conn),
                      pointer(mat_type), pointer(mat_params))
        r = Request(d, pointer(eq), length(dofs), nu, pointer(Uex), pointer(Fex), C_NULL, 0, 0, p)
        rc = ccall((:amr_server_submit, LIB), Cint, (Ptr{Cvoid}, Ref{Request}, Ref{Int64}), srv.h, r, id)
        rc == 0 || error("amr_server_submit failed ($rc)")
    end
    srv.pending[id[]] = (model, dofs)
    return id[]
end

"""
    wait!(srv, id) -> (status, result)

Blocks until request `id` is done and updates its model's dof values as
mech_stage_solver! does; `result` holds the submit, admit and done times.
"""
function wait!(srv::GPUServer, id::Integer)
    model, dofs = pop!(srv.pending, id)
    U = zeros(length(dofs)); F = zeros(length(dofs)); res = RequestResult(); msg = zeros(UInt8, 512)
    rc = ccall((:amr_server_wait, LIB), Cint,
               (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ref{RequestResult}, Ptr{UInt8}, Csize_t),
               srv.h, id, U, F, res, msg, length(msg))
    if rc == 0 || rc == -11
        for (i, dof) in enumerate(dofs)
            dof.vals[dof.name] += U[i]
            dof.vals[dof.natname] += F[i]
        end
    end
    st = rc == 0 ? Amaru.success() : Amaru.failure(unsafe_string(pointer(msg)))
    return st, res
end

# ---------------------------------------------------------------------------
# Handle queries, IP-state checkpoints (src/ip.jl:22-57), per-element E, the
# HBM estimate, server counters and the launch-shape autotuner.
# ---------------------------------------------------------------------------
function checked(g::GPUModel, rc::Integer)
    st = check(g, rc)
    st === nothing || error(st.message)
    return nothing
end

"""
    sizes(g) -> (nnodes, nelems, nip_total, nblocks)

Sizes of the device model (amr_get_sizes); nblocks counts the node blocks of K's pattern.
"""
function sizes(g::GPUModel)
    nn, ne, ni, nb = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0)
    checked(g, ccall((:amr_get_sizes, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ref{Int64}, Ref{Int64}),
                     g.h, nn, ne, ni, nb))
    return (nnodes=nn[], nelems=ne[], nip_total=ni[], nblocks=nb[])
end

"""
    get_state(g) -> Matrix{Float64} (16 x nip_total)

The IP states, one column per IP in element and IP order: σ (6), ε (6), εpa, Δλ and two
zeros, as in the IpState objects of the three materials.
"""
function get_state(g::GPUModel)
    S = zeros(16, sizes(g).nip_total)
    checked(g, ccall((:amr_get_state, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, S))
    return S
end

"""
    set_state!(g, S)

Writes IP states in the layout of get_state: a checkpoint restored, or states set by the caller.
"""
function set_state!(g::GPUModel, S::Matrix{Float64})
    size(S) == (16, sizes(g).nip_total) || error("AmaruGPU: state must be 16 x nip_total")
    checked(g, ccall((:amr_set_state, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, S))
    return g
end

"Backup states ← current states (copyto!.(StateBk, State), src/mech/mech-solver.jl:333)."
commit_state!(g::GPUModel) = (checked(g, ccall((:amr_state_commit, LIB), Cint, (Ptr{Cvoid},), g.h)); g)
"Current states ← backup states (copyto!.(State, StateBk), src/mech/mech-solver.jl:391,461)."
restore_state!(g::GPUModel) = (checked(g, ccall((:amr_state_restore, LIB), Cint, (Ptr{Cvoid},), g.h)); g)

"""
    set_youngs!(g, E)

Young's modulus per element (in element order), replacing the materials' E.
"""
function set_youngs!(g::GPUModel, E::Vector{Float64})
    length(E) == sizes(g).nelems || error("AmaruGPU: one E per element")
    checked(g, ccall((:amr_set_youngs, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), g.h, E))
    return g
end

"""
    estimate_bytes(model::FEModel) -> Int

Upper bound of the device bytes one model and one stage of it take (amr_estimate_bytes),
the figure a GPUServer admits requests by.
"""
function estimate_bytes(model::FEModel)
    coords, shape, nips, conn_ptr, conn, mat_type, mat_params = model_arrays(model)
    ctx = model.ctx
    b = Ref{Int64}(0)
    GC.@preserve coords shape nips conn_ptr conn mat_type mat_params begin
        d = ModelDesc(ctx.ndim, STRESSMODELS[ctx.stressmodel], ctx.thickness, size(coords, 2), pointer(coords),
                      length(shape), pointer(shape), pointer(nips), pointer(conn_ptr), pointer(conn),
                      pointer(mat_type), pointer(mat_params))
        rc = ccall((:amr_estimate_bytes, LIB), Cint, (Ref{ModelDesc}, Ref{Int64}), d, b)
        rc == 0 || error("amr_estimate_bytes failed ($rc)")
    end
    return Int(b[])
end

struct ServerInfo
    queued::Int64; active::Int64; peak_active::Int64; completed::Int64; active_bytes::Int64; peak_bytes::Int64
    seconds::Float64
end

"""
    stats(srv::GPUServer) -> ServerInfo

Queue length, requests on the device (now and at peak), completed requests and the
admitted bytes (now and at peak).
"""
function stats(srv::GPUServer)
    st = Ref{ServerInfo}()
    rc = ccall((:amr_server_stats, LIB), Cint, (Ptr{Cvoid}, Ref{ServerInfo}), srv.h, st)
    rc == 0 || error("amr_server_stats failed ($rc)")
    return st[]
end

struct Tuning
    ngroups::Int32
    shape::NTuple{8,Int32}
    stiffness_epb::NTuple{8,Int32}
    internal_epb::NTuple{8,Int32}
    batch_threads::Int32
    batch_ctas_per_sm::Int32
    stiffness_seconds::Float64
    internal_seconds::Float64
end

"""
    autotune!(g) -> Tuning

Times the candidate launch shapes of the element kernels on this model (and of the batched
solve) and keeps the fastest; needs the DOFs set and changes no result.
"""
function autotune!(g::GPUModel)
    t = Ref{Tuning}()
    checked(g, ccall((:amr_autotune, LIB), Cint, (Ptr{Cvoid}, Ref{Tuning}), g.h, t))
    return t[]
end

# ---------------------------------------------------------------------------
# Coupled mounts: hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) and
# tm_mount_global_matrices (src/thermomech/thermomech-solver.jl:80-170) on the device.
# ---------------------------------------------------------------------------
struct CoupledDesc
    kind::Int32; pad::Int32
    gammaw::Float64; T0::Float64
    params::Ptr{Float64}
end

function coupled_mount(model::FEModel, ndofs::Int, Δt::Float64, kind::Int32, key::Symbol)
    g = gpu_model!(model)            # the active elements (the mounts loop over active_elems)
    nn = length(g.nodes)
    eq4 = fill(Int64(-1), 4, nn)     # ux, uy, uz, the scalar; 0-based, device node order
    phi = zeros(ndofs)               # dof.vals of the scalar DOFs, as the reference reads them
    for (i, id) in enumerate(g.nodes)
        node = model.nodes[id]
        for (c, k) in enumerate((:ux, :uy, :uz))
            haskey(node.dofdict, k) && (eq4[c, i] = node.dofdict[k].eq_id - 1)
        end
        if haskey(node.dofdict, key)
            dof = node.dofdict[key]
            eq4[4, i] = dof.eq_id - 1
            phi[dof.eq_id] = dof.vals[key]
        end
    end
    prm = zeros(3, length(g.elems))
    for (k, e) in enumerate(g.elems)
        if kind == 0  # HMSolid: Biot's alpha, permeability, storativity (LinearElasticSeep)
            prm[:, k] .= (e.props.α, e.mat.k, e.mat.S)
        else          # TMSolid: thermal expansion, conductivity (LinearElasticThermo), rho cv
            prm[:, k] .= (e.props.α, e.mat.k, e.props.ρ * e.props.cv)
        end
    end
    nnz = Ref{Int64}(0)
    local colptr, rowval, nzval, rhs
    GC.@preserve prm eq4 phi begin
        d = CoupledDesc(kind, 0, kind == 0 ? model.ctx.γw : 0.0, kind == 1 ? model.ctx.T0 : 0.0, pointer(prm))
        checked(g, ccall((:amr_coupled_mount, LIB), Cint, (Ptr{Cvoid}, Ref{CoupledDesc}, Ptr{Int64}, Int64, Float64,
                         Ptr{Float64}, Ref{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
                         g.h, d, eq4, ndofs, Δt, phi, nnz, C_NULL, C_NULL, C_NULL, C_NULL))
        colptr = zeros(Int64, ndofs + 1); rowval = zeros(Int64, nnz[]); nzval = zeros(nnz[]); rhs = zeros(ndofs)
        checked(g, ccall((:amr_coupled_mount, LIB), Cint, (Ptr{Cvoid}, Ref{CoupledDesc}, Ptr{Int64}, Int64, Float64,
                         Ptr{Float64}, Ref{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
                         g.h, d, eq4, ndofs, Δt, phi, nnz, colptr, rowval, nzval, rhs))
    end
    return SparseMatrixCSC(ndofs, ndofs, colptr .+ 1, rowval .+ 1, nzval), rhs
end

"""
    gpu_hm_mount_global_matrices(model, ndofs, Δt)

hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) on the device for HMSolid elements with
LinearElasticSeep: (G, RHS) with every element entry and the reference's summation order.
"""
gpu_hm_mount_global_matrices(model::FEModel, ndofs::Int, Δt::Float64) = coupled_mount(model, ndofs, Δt, Int32(0), :uw)

"""
    gpu_tm_mount_global_matrices(model, ndofs, Δt)

tm_mount_global_matrices (src/thermomech/thermomech-solver.jl:80-170) on the device for TMSolid elements with
LinearElasticThermo: (G, RHS).
"""
gpu_tm_mount_global_matrices(model::FEModel, ndofs::Int, Δt::Float64) = coupled_mount(model, ndofs, Δt, Int32(1), :ut)

export GPUModel, solve_gpu!, gpu_stage_solver!, GPUBatch, solve_batch!, GPUServer, submit!, wait!,
       nodal_patch_recovery_gpu, has_gpu, gpu_dyn_stage_solver!, gpu_modal_solver!, save_gpu,
       sizes, get_state, set_state!, commit_state!, restore_state!, set_youngs!, estimate_bytes, stats, autotune!,
       rayleigh_coefficients, gpu_hm_mount_global_matrices, gpu_tm_mount_global_matrices, set_amg_smoothing!

end # module
