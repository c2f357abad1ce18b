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
# library does not support raise an error: there is no CPU fallback.
#
# Index convention: the C ABI is 0-based; this file converts (eq_id - 1).
module AmaruGPU

using Amaru
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
material_code(m) = error("AmaruGPU: material $(typeof(m)) is not on the GPU path")

"""
    GPUModel(model::FEModel)

Creates the device model: nodes, MechSolid elements with their material
parameters and quadrature, pattern and contribution map (amr_model_create).
"""
function GPUModel(model::FEModel)
    elems = model.elems
    all(e -> e isa MechSolid, elems) || error("AmaruGPU: only MechSolid elements are on the GPU path")
    nnodes = length(model.nodes)
    coords = zeros(3, nnodes)
    for (i, n) in enumerate(model.nodes)
        coords[:, i] .= (n.coord.x, n.coord.y, n.coord.z)
    end
    nel = length(elems)
    shape = Int32[SHAPES[e.shape.name] for e in elems]
    nips = Int32[length(e.ips) for e in elems]
    conn_ptr = zeros(Int64, nel + 1)
    conn = Int64[]
    mat_type = zeros(Int32, nel)
    mat_params = zeros(8, nel)
    for (k, e) in enumerate(elems)
        append!(conn, [n.id - 1 for n in e.nodes])
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
    g = GPUModel(h[], 0, 0)
    finalizer(x -> ccall((:amr_model_destroy, LIB), Cint, (Ptr{Cvoid},), x.h), g)
    return g
end

"""
    set_dofs!(g, model, dofs, nu)

Passes the numbering of configure_dofs! (src/bc.jl:198-233) to the library.
"""
function set_dofs!(g::GPUModel, model::FEModel, dofs, nu)
    eq = fill(Int64(-1), 3, length(model.nodes))
    keys = (:ux, :uy, :uz)
    for n in model.nodes
        for (k, key) in enumerate(keys)
            haskey(n.dofdict, key) && (eq[k, n.id] = n.dofdict[key].eq_id - 1)
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

"""
    gpu_stage_solver!(ana::MechAnalysis, stage::Stage; args...)

mech_stage_solver! with the Newton loop, K, the solves and the IP states on
the device.  The essential values and loads come from Amaru's own
configure_dofs! and get_bc_vals; the dof values are updated as the reference
does (src/mech/mech-solver.jl:394-397).
"""
function gpu_stage_solver!(ana::MechAnalysis, stage::Stage; args...)
    args = NamedTuple(args)
    model = ana.model
    g = get!(() -> GPUModel(model), GPU_MODELS, objectid(model))
    dofs, nu = Amaru.configure_dofs!(model, stage.bcs)
    model.ndofs = length(dofs)
    set_dofs!(g, model, dofs, nu)
    Uex, Fex = Amaru.get_bc_vals(model, stage.bcs)
    scheme = Dict(:FE => 0, :ME => 1, :BE => 2, :Ralston => 3)[Symbol(args.scheme)]
    lin = SolveOpts(0, 1e-8, 20000, 32)
    p = StageParams(args.tol, args.rtol, args.rspan, args.dT0, args.dTmin, args.dTmax, scheme, args.maxits,
                    args.autoinc, stage.nincs, stage.nouts, lin)
    U = zeros(length(dofs))
    F = zeros(length(dofs))
    stats = StageStats()
    rc = ccall((:amr_stage_run, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{StageParams}, Ptr{Float64}, Ptr{Float64}, Ref{StageStats}),
               g.h, Uex, Fex, p, U, F, stats)
    if rc == 0 || rc == -11
        for (i, dof) in enumerate(dofs)
            dof.vals[dof.name] += U[i]
            dof.vals[dof.natname] += F[i]
        end
    end
    rc == 0 && return Amaru.success()
    return check(g, rc)
end

const GPU_MODELS = Dict{UInt,GPUModel}()

"""
    solve_gpu!(ana::MechAnalysis; args...)

solve! with the stage solver replaced by gpu_stage_solver!.
"""
function solve_gpu!(ana::MechAnalysis; args...)
    args = Amaru.checkargs(args, Amaru.mech_solver_params)
    return Amaru.stage_iterator!(gpu_stage_solver!, ana; args...)
end

export GPUModel, solve_gpu!, gpu_stage_solver!

end # module
