classdef SGPEtaskGB300 < GPEtaskGB300
    %SGPEtaskGB300 - SGPEtask (stochastic GPE) whose solve_split runs on a
    %GB300 GPU through libgpe (gpe_mex 'sgpe' -> gpe_solve_sgpe).
    %
    % Properties as SGPEtask (T, ecut, snapshots, ss_maxlength) plus seed, the
    % key of the counter-based noise stream (MATLAB's global randn stream is
    % not used, so a run is reproducible from its seed).  groundstate_itp and
    % get_energy are the GPEtaskGB300 ones.  A scalar omega runs the rotating
    % SGPE (its Lz Crank-Nicolson step, solve_split.m:58-64).  As in SGPEtask,
    % a user_callback that returns 'TERM' ends the run after that outer step
    % (solve_split.m:77-80).
    %
    % UNVERIFIED: no MATLAB was available where this file was written; the
    % library call it makes is covered by the Python tests of the same ABI.

    properties
        T = 0               % temperature
        snapshots = {}      % kept for SGPEtask compatibility
        ss_maxlength = 100
        ecut = 0            % cut-off energy (applies when T > 0)
        seed = 0            % noise stream key (64-bit integer value)
    end

    methods
        function obj = SGPEtaskGB300(grid, trappot)
            obj@GPEtaskGB300(grid, trappot);
        end

        function phi = solve_split(task, ddt, niter_inner, niter_outer)
            % @SGPEtask/solve_split.m semantics, executed by libgpe.
            task.dispstat('', 'init');
            tic;
            task.gb300_push();
            if task.current_iter > 0
                phi = task.current_state;
            else
                phi = task.init_state;
            end
            gpe_mex('set_state', task.gb300_handle, complex(gather(phi)));
            timedep = isa(task.Vtd, 'function_handle') || numel(task.V0) > 1;
            if ~timedep
                gpe_mex('set_potential', task.gb300_handle, double(gather(task.Vtrap)));
            end
            gpe_mex('sgpe', task.gb300_handle, ddt, niter_inner, niter_outer, task, timedep, ...
                double(task.T), double(task.ecut), double(task.seed));
            phi = task.current_state;
        end

        function stop = gb300_step(task, step, time, mu, n)
            % Called by the gateway after each outer step; nonzero ends the run.
            res = task.ext_callback(task.gb300_state(), step, time, mu, n);
            stop = double(ischar(res) && strcmp(res, 'TERM'));
        end
    end

    methods (Access = protected)
        function res = ext_callback(obj, phi, step, time, mu, n)
            % SGPEtask.m:20-44: the bookkeeping of GPEtask.ext_callback, and the
            % user callback's text is returned (solve_split.m:77 tests it).
            obj.current_state = phi;
            obj.current_time = time;
            obj.current_iter = step;
            obj.current_mu = mu;
            obj.history.mu(step) = mu;
            obj.current_n = n;
            obj.history.n(step) = n;
            res = '';
            if isa(obj.user_callback, 'function_handle')
                if nargout(obj.user_callback) ~= 0
                    res = obj.user_callback(obj);
                else
                    obj.user_callback(obj);
                end
            end
            obj.dispstat(sprintf(['Split-step: iter - %u, mu - %0.3f, calc. time - %0.3f sec.; ', res], ...
                step, mu, toc));
        end
    end
end
